"""The small-image objective as one cooperative launch (k_objective_fused)
against the same passes as separate launches (GV_FUSED=0): chi2, the
residuals, the objective with its priors, and whole frprmn / L-BFGS solves
agree bit for bit, including the plain-MEM 256^2 configuration (104,400
visibilities) solved for 100 frprmn iterations."""

import os

import numpy as np
import pytest

from gpuvmem_gb300 import synth

pytestmark = pytest.mark.gpu

TERMS = [("Chi2", 1.0), ("Entropy", 0.01), ("TotalSquaredVariation", 1e-5)]


def _problem(fused, cfg, terms=TERMS):
    import gpuvmem_gb300 as gv
    os.environ["GV_FUSED"] = "1" if fused else "0"
    try:
        data = synth.generate(cfg, device="cuda")
        return gv.Problem(data, [gv.term(k, lam) for k, lam in terms])
    finally:
        os.environ.pop("GV_FUSED", None)


def _image(prob, seed):
    import torch
    rng = np.random.default_rng(seed)
    img = prob.initial_image().cpu().numpy()
    img[0] += ((rng.uniform(0, 1, img[0].shape) < 0.1) *
               np.abs(rng.normal(0, 2000.0, img[0].shape))).astype(np.float32)
    img[1] = rng.uniform(-1, 3, img[1].shape).astype(np.float32)
    return torch.from_numpy(img).cuda()


@pytest.mark.parametrize("n,nchan", [(64, 2), (256, 1), (512, 1)])
def test_fused_objective_bit_identical(n, nchan):
    cfg = synth.small_config(n=n, n_ant=10, n_times=48, nchan=nchan, seed=60 + n)
    pa, pb = _problem(True, cfg), _problem(False, cfg)
    for flag in (0, 1):
        img = _image(pa, 3 + flag)
        da, db = img.clone(), img.clone()
        ca, cb = pa.chi2(da, flag), pb.chi2(db, flag)
        assert np.float64(ca).tobytes() == np.float64(cb).tobytes(), (ca, cb)
        np.testing.assert_array_equal(da.cpu().numpy().view(np.uint32),
                                      db.cpu().numpy().view(np.uint32))
        np.testing.assert_array_equal(pa.residuals().view(np.uint32),
                                      pb.residuals().view(np.uint32))
        pa.set_iteration(1)
        pb.set_iteration(1)
        da, db = img.clone(), img.clone()
        fa, fia = pa.objective(da, flag)
        fb, fib = pb.objective(db, flag)
        assert np.float64(fa).tobytes() == np.float64(fb).tobytes(), (fa, fb)
        assert np.array(fia).tobytes() == np.array(fib).tobytes(), (fia, fib)
        np.testing.assert_array_equal(da.cpu().numpy().view(np.uint32),
                                      db.cpu().numpy().view(np.uint32))
        pa.set_iteration(0)
        pb.set_iteration(0)


@pytest.mark.parametrize("method,iterations,terms", [
    ("CG-FRPRMN", 12, TERMS),
    ("CG-LBFGS", 10, TERMS),
    ("CG-FRPRMN", 10, TERMS + [("L1-Norm", 1e-4), ("TotalVariation", 1e-5)]),
])
def test_fused_solves_bit_identical(method, iterations, terms):
    import torch
    cfg = synth.small_config(n=64, nchan=2, seed=21)
    out = []
    for fused in (True, False):
        prob = _problem(fused, cfg, terms)
        img = prob.initial_image()
        rep = prob.optimize(img, method, iterations=iterations)
        torch.cuda.synchronize()
        out.append((rep, img.cpu().numpy()))
        prob.close()
    (ra, ia), (rb, ib) = out
    assert ra.iterations == rb.iterations and ra.n_objective == rb.n_objective
    assert np.float32(ra.f_final).tobytes() == np.float32(rb.f_final).tobytes()
    np.testing.assert_array_equal(ia.view(np.uint32), ib.view(np.uint32))


def test_fused_plain256_frprmn_trajectory():
    """The plain-MEM 256^2 configuration (chi2 + entropy 0.01), frprmn for
    100 iterations: the same iterations, evaluations, objective and image
    bit for bit with and without the fused launch."""
    import torch
    out = []
    for fused in (True, False):
        prob = _problem(fused, synth.CONFIG0, [("Chi2", 1.0), ("Entropy", 0.01)])
        img = prob.initial_image()
        rep = prob.optimize(img, "CG-FRPRMN", iterations=100)
        torch.cuda.synchronize()
        out.append((rep, img.cpu().numpy()))
        prob.close()
    (ra, ia), (rb, ib) = out
    print(f"\nplain 256^2 frprmn: {ra.iterations} iterations, {ra.n_objective} objective "
          f"evaluations, f = {ra.f_final!r}; fused {ra.seconds * 1e3:.1f} ms, "
          f"separate launches {rb.seconds * 1e3:.1f} ms")
    assert ra.iterations == rb.iterations and ra.n_objective == rb.n_objective
    assert np.float32(ra.f_final).tobytes() == np.float32(rb.f_final).tobytes()
    np.testing.assert_array_equal(ia.view(np.uint32), ib.view(np.uint32))
