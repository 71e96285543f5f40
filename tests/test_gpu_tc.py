"""Tensor-core DChi2 engine (tcgen05) against the FP64 oracle and the exact
SIMT engine, through the C ABI."""

import numpy as np
import pytest

import oracle as O
from gpuvmem_gb300 import synth

pytestmark = pytest.mark.gpu

GRAD_TOL = 1e-5
TERMS = [(O.FI_CHI2, 1.0, 0, 0, 0.0, 0.0, 0.0), (O.FI_ENTROPY, 0.01, 0, 0, 0.001, -1.0, 0.0)]


def build(n, nchan, seed, engine):
    import gpuvmem_gb300 as gv
    cfg = synth.small_config(n=n, n_ant=10, n_times=48, nchan=nchan, seed=seed)
    data = synth.generate(cfg)
    orc = O.Oracle(data, TERMS)
    prob = gv.Problem(data, TERMS, engine=engine)
    return data, orc, prob


def image(orc, seed, alpha=False):
    rng = np.random.default_rng(seed)
    img = orc.initial_image()
    img[0] += ((rng.uniform(0, 1, img[0].shape) < 0.1) *
               np.abs(rng.normal(0, 3000.0, img[0].shape))).astype(np.float32)
    if alpha:
        img[1] = rng.uniform(-1, 3, img[1].shape).astype(np.float32)
    return img


@pytest.mark.parametrize("n,nchan", [(128, 1), (256, 2)])
def test_tc_engine_selected_and_matches_oracle(n, nchan):
    import torch
    data, orc, prob = build(n, nchan, 40 + n, engine=2)
    assert prob.info.dchi2_engine == 2
    img = image(orc, 3)
    _, img_c = orc.chi2(img.copy())
    ref = orc.dchi2(img_c)
    d = torch.from_numpy(img.copy()).cuda()
    prob.chi2(d)
    got = prob.dchi2(d).cpu().numpy()
    err = np.abs(got - ref).max() / np.abs(ref[0]).max()
    assert err <= GRAD_TOL, err


def test_tc_matches_simt_channels_and_dirty():
    import torch
    data, orc, p2 = build(256, 2, 77, engine=2)
    import gpuvmem_gb300 as gv
    p1 = gv.Problem(data, TERMS, engine=1)
    img = image(orc, 5)
    d1 = torch.from_numpy(img.copy()).cuda()
    d2 = torch.from_numpy(img.copy()).cuda()
    p1.chi2(d1)
    p2.chi2(d2)
    for c in range(2):
        a = p1.dchi2_channel(c).cpu().numpy()
        b = p2.dchi2_channel(c).cpu().numpy()
        assert np.abs(a - b).max() <= 2 * GRAD_TOL * np.abs(a).max()
    a = p1.dirty_image().cpu().numpy()
    b = p2.dirty_image().cpu().numpy()
    assert np.abs(a - b).max() <= 2 * GRAD_TOL * np.abs(a).max()
    a = p1.psf_image().cpu().numpy()
    b = p2.psf_image().cpu().numpy()
    assert np.abs(a - b).max() <= 2 * GRAD_TOL * np.abs(a).max()


def test_tc_alpha_plane():
    import torch
    data, orc, prob = build(128, 2, 91, engine=2)
    img = image(orc, 8, alpha=True)
    _, img_c = orc.chi2(img.copy(), flag_opt=1)
    ref = orc.dchi2(img_c, flag_opt=1)
    d = torch.from_numpy(img.copy()).cuda()
    prob.chi2(d, 1)
    got = prob.dchi2(d, 1).cpu().numpy()
    mag = np.zeros_like(ref[1])
    for c in range(len(data.freqs)):
        nud = np.float64(np.float32(data.freqs[c]) / np.float32(data.nu_0))
        mag += np.abs(orc.dchi2_channel(c) * img_c[0] * nud ** img_c[1] * orc.fg_scale * np.log(nud))
    assert np.abs(got - ref).max() <= GRAD_TOL * mag.max()


@pytest.mark.parametrize("env", [{"GV_TC_PAIR": "0"}, {"GV_TC_SLAB": "1"},
                                 {"GV_TC_ACCURATE_ANCHOR": "1"}, {"GV_TC_PARTS": "2"},
                                 {"GV_TC_PAIR": "0", "GV_TC_PARTS": "2", "GV_TC_SLAB": "3"}])
def test_tc_launch_variants_match_simt(env, monkeypatch):
    """CTA pairs (cta_group::2) and single CTAs, one or two accumulator parts,
    the drain period and the anchor phasor's sin/cos give the same gradient
    as the exact SIMT engine."""
    import torch
    import gpuvmem_gb300 as gv
    data, orc, _ = build(512, 3, 123, engine=1)
    p1 = gv.Problem(data, TERMS, engine=1)
    img = image(orc, 9)
    d1 = torch.from_numpy(img.copy()).cuda()
    p1.chi2(d1)
    ref = p1.dchi2(d1).cpu().numpy()
    for k, v in env.items():
        monkeypatch.setenv(k, v)
    p2 = gv.Problem(data, TERMS, engine=2)
    d2 = torch.from_numpy(img.copy()).cuda()
    p2.chi2(d2)
    got = p2.dchi2(d2).cpu().numpy()
    monkeypatch.undo()
    got_default = p2.dchi2(d2).cpu().numpy()
    scale = np.abs(ref[0]).max()
    assert np.abs(got - ref).max() <= GRAD_TOL * scale
    assert np.abs(got_default - ref).max() <= GRAD_TOL * scale
