"""The line search on the GPU (bracket + Brent as a state machine inside a
CUDA-graph WHILE loop, one graph launch per linmin) and the L-BFGS recursion
with its scalars on the GPU, against the host versions: the same points and
the same scalars, so iterations, evaluation counts, the final objective and
the image agree bit for bit."""

import os

import numpy as np
import pytest

from gpuvmem_gb300 import synth

pytestmark = pytest.mark.gpu


def _solve(device_ls, method, iterations, seed, n=64, nchan=1, device_lbfgs=True, terms=None):
    import torch
    import gpuvmem_gb300 as gv
    os.environ["GV_DEVICE_LS"] = "1" if device_ls else "0"
    os.environ["GV_DEVICE_LBFGS"] = "1" if device_lbfgs else "0"
    try:
        data = synth.generate(synth.small_config(n=n, nchan=nchan, seed=seed), device="cuda")
        terms = terms or [("Chi2", 1.0), ("Entropy", 0.01), ("TotalSquaredVariation", 1e-5)]
        prob = gv.Problem(data, [gv.term(k, lam) for k, lam in terms])
        img = prob.initial_image()
        rep = prob.optimize(img, method, iterations=iterations)
        torch.cuda.synchronize()
        return rep, img.cpu().numpy()
    finally:
        os.environ.pop("GV_DEVICE_LS", None)
        os.environ.pop("GV_DEVICE_LBFGS", None)


@pytest.mark.parametrize("method,iterations", [("CG-FRPRMN", 15), ("CG-LBFGS", 10)])
def test_device_line_search_matches_host(method, iterations):
    rh, ih = _solve(False, method, iterations, seed=21)
    rd, idv = _solve(True, method, iterations, seed=21)
    assert rd.iterations == rh.iterations and rd.exit_reason == rh.exit_reason
    assert rd.n_objective == rh.n_objective and rd.n_gradient == rh.n_gradient
    assert np.float32(rd.f_final).tobytes() == np.float32(rh.f_final).tobytes()
    np.testing.assert_array_equal(idv.view(np.uint32), ih.view(np.uint32))


def test_device_line_search_two_channels_128():
    rh, ih = _solve(False, "CG-FRPRMN", 8, seed=5, n=128, nchan=2)
    rd, idv = _solve(True, "CG-FRPRMN", 8, seed=5, n=128, nchan=2)
    assert rd.n_objective == rh.n_objective
    np.testing.assert_array_equal(idv.view(np.uint32), ih.view(np.uint32))


def test_device_line_search_three_priors():
    """Three priors in one prior kernel that forms xt itself (clip2IWNoise
    applied, as Chi2 comes first) and runs beside the Chi2 kernels."""
    terms = [("Chi2", 1.0), ("Entropy", 0.01), ("TotalSquaredVariation", 1e-5), ("L1-Norm", 1e-4)]
    rh, ih = _solve(False, "CG-FRPRMN", 10, seed=9, terms=terms)
    rd, idv = _solve(True, "CG-FRPRMN", 10, seed=9, terms=terms)
    assert rd.iterations == rh.iterations and rd.n_objective == rh.n_objective
    assert np.float32(rd.f_final).tobytes() == np.float32(rh.f_final).tobytes()
    np.testing.assert_array_equal(idv.view(np.uint32), ih.view(np.uint32))


@pytest.mark.parametrize("n", [64, 256])
def test_device_lbfgs_recursion_matches_host(n):
    rh, ih = _solve(True, "CG-LBFGS", 12, seed=23, n=n, device_lbfgs=False)
    rd, idv = _solve(True, "CG-LBFGS", 12, seed=23, n=n, device_lbfgs=True)
    assert rd.iterations == rh.iterations and rd.n_objective == rh.n_objective
    assert np.float32(rd.f_final).tobytes() == np.float32(rh.f_final).tobytes()
    np.testing.assert_array_equal(idv.view(np.uint32), ih.view(np.uint32))
