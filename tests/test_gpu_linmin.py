"""gv_linmin, the C-ABI counterpart of the reference's linmin
(src/linmin.cu:52-110): the bracket + Brent search along a direction on the
GPU (a CUDA-graph WHILE loop) against the host search (GV_DEVICE_LS=0) --
the same minimum, evaluation count, point and direction bit for bit -- and
newP's update of the point and the direction."""

import os

import numpy as np
import pytest

from gpuvmem_gb300 import synth

pytestmark = pytest.mark.gpu

TERMS = [("Chi2", 1.0), ("Entropy", 0.01), ("TotalSquaredVariation", 1e-5)]


def _linmin(device_ls, cfg, iteration, seed):
    import torch
    import gpuvmem_gb300 as gv
    os.environ["GV_DEVICE_LS"] = "1" if device_ls else "0"
    try:
        data = synth.generate(cfg, device="cuda")
        prob = gv.Problem(data, [gv.term(k, lam) for k, lam in TERMS])
    finally:
        os.environ.pop("GV_DEVICE_LS", None)
    img = prob.initial_image()
    rng = np.random.default_rng(seed)
    base = img.cpu().numpy()
    base[0] += np.abs(rng.normal(0.0, 0.01, base[0].shape)).astype(np.float32)
    p = torch.from_numpy(base).cuda()
    xi = prob.gradient(p, 1)
    prob.set_iteration(iteration)
    d = -xi
    p0, d0 = p.clone(), d.clone()
    fret, evals = prob.linmin(p, d)
    torch.cuda.synchronize()
    out = (fret, evals, p.cpu().numpy(), d.cpu().numpy(), p0.cpu().numpy(), d0.cpu().numpy())
    prob.close()
    return out


@pytest.mark.parametrize("n,nchan,iteration", [(64, 1, 0), (64, 2, 1), (256, 1, 1)])
def test_linmin_device_matches_host(n, nchan, iteration):
    cfg = synth.small_config(n=n, n_ant=12, n_times=40, nchan=nchan, seed=80 + n + nchan)
    fd, kd, pd, dd, p0, d0 = _linmin(True, cfg, iteration, seed=5)
    fh, kh, ph, dh, _, _ = _linmin(False, cfg, iteration, seed=5)
    assert kd == kh and kd > 3
    assert np.float32(fd).tobytes() == np.float32(fh).tobytes()
    np.testing.assert_array_equal(pd.view(np.uint32), ph.view(np.uint32))
    np.testing.assert_array_equal(dd.view(np.uint32), dh.view(np.uint32))
    # newP (src/functions.cu:2760-2777): d <- xmin d and p <- p + d where
    # that stays above the floor; elsewhere p = the floor and d = 0
    moved = (dd[0] != 0) & (d0[0] != 0)
    floored = (dd[0] == 0) & (d0[0] != 0)
    assert moved.sum() + floored.sum() > 100
    if moved.any():
        xmin = (dd[0][moved] / d0[0][moved]).astype(np.float64)
        assert np.allclose(xmin, np.median(xmin), rtol=1e-5)
        np.testing.assert_array_equal(pd[0][moved], (p0[0] + dd[0])[moved])
    if floored.any():
        assert np.unique(pd[0][floored]).size == 1
