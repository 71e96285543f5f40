"""CUDA-graph replay of evaluations: gv_evaluate against gv_objective +
gv_gradient, and the optimiser with and without graphs."""

import numpy as np
import pytest

from gpuvmem_gb300 import synth

pytestmark = pytest.mark.gpu

TERMS = None


def _problem(n=128, nchan=2, seed=11):
    import gpuvmem_gb300 as gv
    data = synth.generate(synth.small_config(n=n, nchan=nchan, seed=seed))
    terms = [gv.term("Chi2", 1.0), gv.term("Entropy", 0.01), gv.term("TotalSquaredVariation", 1e-4)]
    return data, terms


def _image(prob, seed):
    import torch
    rng = np.random.default_rng(seed)
    img = prob.initial_image().cpu().numpy()
    img[0] += ((rng.uniform(0, 1, img[0].shape) < 0.1) *
               np.abs(rng.normal(0, 1000.0, img[0].shape))).astype(np.float32)
    return torch.from_numpy(img).cuda()


def test_evaluate_matches_objective_then_gradient():
    import torch
    import gpuvmem_gb300 as gv
    data, terms = _problem()
    pa = gv.Problem(data, terms)
    pb = gv.Problem(data, terms)
    for step, it in enumerate([0, 0, 1, 2, 1]):
        img = _image(pa, 100 + step % 2)
        ia, ib = img.clone(), img.clone()
        xa = torch.zeros_like(img)
        xb = torch.zeros_like(img)
        n0 = gv.launch_count()
        fa, fia, _ = pa.evaluate(ia, it, xi=xa)
        n1 = gv.launch_count()
        fb, fib = pb.objective(ib)
        pb.gradient(ib, it, xi=xb)
        n2 = gv.launch_count()
        assert fa == fb and fia == fib, (step, fa, fb)
        assert torch.equal(ia, ib)  # the clip written back into the image
        assert torch.equal(xa, xb)
        assert n1 - n0 == n2 - n1 > 0  # replays count their kernels


def test_gradient_graph_matches_direct_launches():
    """gv_gradient replays a captured gradient (factor pass, DChi2 GEMM,
    split-K reduction, prior gradients) when graphs are on; the result is
    the launch-by-launch one bit for bit, at both gating states."""
    import torch
    import gpuvmem_gb300 as gv
    data, terms = _problem(n=256, nchan=2, seed=13)
    pa = gv.Problem(data, terms)
    pb = gv.Problem(data, terms)
    pb.set_graphs(False)
    for step, it in enumerate([0, 1, 2]):
        img = _image(pa, 200 + step)
        ia, ib = img.clone(), img.clone()
        xa = torch.zeros_like(img)
        xb = torch.zeros_like(img)
        pa.objective(ia)
        pb.objective(ib)
        pa.gradient(ia, it, xi=xa)
        pb.gradient(ib, it, xi=xb)
        assert torch.equal(xa, xb), step


def test_objective_many_matches_objective():
    """gv_objective_many scores a list of images with one synchronisation;
    each value equals gv_objective's, and the listed images stay unclipped."""
    import torch
    import gpuvmem_gb300 as gv
    data, terms = _problem(n=128, nchan=2, seed=17)
    pa = gv.Problem(data, terms)
    pa.set_iteration(1)
    imgs = torch.stack([_image(pa, 300 + k) for k in range(5)])
    before = imgs.clone()
    fm = pa.objective_many(imgs)
    assert torch.equal(imgs, before)
    for k in range(imgs.shape[0]):
        f, _ = pa.objective(imgs[k].clone())
        assert fm[k] == f, (k, fm[k], f)


@pytest.mark.parametrize("method", ["CG-FRPRMN", "CG-LBFGS"])
def test_optimizer_with_and_without_graphs(method):
    import gpuvmem_gb300 as gv
    data, terms = _problem(n=64, nchan=1, seed=5)
    pa = gv.Problem(data, terms)
    pb = gv.Problem(data, terms)
    pb.set_graphs(False)
    ia = pa.initial_image()
    ib = pb.initial_image()
    ra = pa.optimize(ia, method=method, iterations=4)
    rb = pb.optimize(ib, method=method, iterations=4)
    assert ra.f_final == rb.f_final and ra.iterations == rb.iterations
    assert ra.n_objective == rb.n_objective
    import torch
    assert torch.equal(ia, ib)
