"""Autotuner: the kept launch shapes are valid, no slower than the defaults
on the measured problem, and the results stay at the engine's parity with
the FP64 oracle."""

import numpy as np
import pytest

import oracle as O
from gpuvmem_gb300 import synth

pytestmark = pytest.mark.gpu

TERMS = [(O.FI_CHI2, 1.0, 0, 0, 0.0, 0.0, 0.0), (O.FI_ENTROPY, 0.01, 0, 0, 0.001, -1.0, 0.0)]


@pytest.mark.parametrize("n", [128, 256])
def test_autotune_keeps_parity(n):
    import torch
    import gpuvmem_gb300 as gv
    cfg = synth.small_config(n=n, n_ant=10, n_times=48, nchan=2, seed=70 + n)
    data = synth.generate(cfg)
    orc = O.Oracle(data, TERMS)
    prob = gv.Problem(data, TERMS, engine=2)
    r = prob.autotune()
    assert r.tc_pair in (0, 1) and r.tc_nsplit >= 1 and r.candidates >= 6
    assert r.degrid_threads in (128, 256) and r.degrid_blocks >= 1
    assert r.dchi2_ms_tuned <= r.dchi2_ms_default * 1.05
    assert r.chi2_ms_tuned <= r.chi2_ms_default * 1.05
    rng = np.random.default_rng(4)
    img = orc.initial_image()
    img[0] += ((rng.uniform(0, 1, img[0].shape) < 0.1) *
               np.abs(rng.normal(0, 3000.0, img[0].shape))).astype(np.float32)
    c_ref, img_c = orc.chi2(img.copy())
    g_ref = orc.dchi2(img_c)
    d = torch.from_numpy(img.copy()).cuda()
    c = prob.chi2(d)
    g = prob.dchi2(d).cpu().numpy()
    assert abs(c - c_ref) <= 1e-5 * abs(c_ref)
    assert np.abs(g - g_ref).max() <= 1e-5 * np.abs(g_ref[0]).max()
