"""Batches of independent problems: one graph launch (and the kernel-by-
kernel path) give each problem exactly what gv_objective + gv_gradient give
it alone."""

import numpy as np
import pytest

from gpuvmem_gb300 import synth

pytestmark = pytest.mark.gpu


def _setup(sizes):
    import gpuvmem_gb300 as gv
    datas, terms = [], []
    for k, n in enumerate(sizes):
        datas.append(synth.generate(synth.small_config(n=n, nchan=1 + k % 2, seed=50 + k)))
        terms.append([gv.term("Chi2", 1.0), gv.term("Entropy", 0.01 * (k + 1)),
                      gv.term("TotalSquaredVariation", 1e-4)])
    return datas, terms


def _image(prob, seed):
    import torch
    rng = np.random.default_rng(seed)
    img = prob.initial_image().cpu().numpy()
    img[0] += ((rng.uniform(0, 1, img[0].shape) < 0.1) *
               np.abs(rng.normal(0, 1000.0, img[0].shape))).astype(np.float32)
    return torch.from_numpy(img).cuda()


@pytest.mark.parametrize("graphs,fused", [(True, False), (True, True), (False, False)])
def test_batch_matches_single_problems(graphs, fused, monkeypatch):
    """fused: the objectives of all problems as one cooperative launch over
    an offset table of their tasks (GV_BATCH_FUSED=1)."""
    import torch
    import gpuvmem_gb300 as gv
    datas, terms = _setup([64, 128, 128, 256, 64, 512])
    pa = [gv.Problem(d, t) for d, t in zip(datas, terms)]
    pb = [gv.Problem(d, t) for d, t in zip(datas, terms)]
    monkeypatch.setenv("GV_BATCH_FUSED", "1" if fused else "0")
    batch = gv.Batch(pa)
    monkeypatch.undo()
    batch.set_graphs(graphs)
    imgs0 = [_image(p, 7 + i) for i, p in enumerate(pa)]
    for it in (0, 1, 2, 2):
        ia = [x.clone() for x in imgs0]
        ib = [x.clone() for x in imgs0]
        xa = [torch.zeros_like(x) for x in ia]
        xb = [torch.zeros_like(x) for x in ib]
        fa = batch.evaluate(ia, xa, it)
        for p, i_, x_, f in zip(pb, ib, xb, fa):
            fb, _ = p.objective(i_)
            p.gradient(i_, it, xi=x_)
            assert f == fb
        for u, v in zip(ia, ib):
            assert torch.equal(u, v)
        for u, v in zip(xa, xb):
            assert torch.equal(u, v)
