"""The CPU oracle pinned against golden outputs of the reference's own CUDA
kernels (tests/golden/*.npz, written by tests/golden/make_golden.py on a
GB300 through the reference harness).  Runs without a GPU."""

import glob
import os
import types

import numpy as np
import pytest

import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "ref_*.npz")))
TERMS = [(O.FI_CHI2, 1.0, 0, 0, 0.0, 0.0, 0.0)]
PRIOR_TERMS = {1: (O.FI_ENTROPY, 0.01, 0, 0, 0.001, -1.0, 0.0),
               2: (O.FI_TSV, 1e-4, 0, 0, 0.0, 0.0, 0.0),
               3: (O.FI_TV, 1e-4, 0, 0, 0.0, 0.0, 1e-12),
               4: (O.FI_L1, 1e-3, 0, 0, 0.0, 0.0, 1e-12),
               5: (O.FI_LAPLACIAN, 1e-5, 0, 0, 0.0, 0.0, 0.0)}


def load(path):
    z = np.load(path)
    d = types.SimpleNamespace(**{k: z[k] for k in z.files})
    for k in ["M", "N", "primary_beam"]:
        setattr(d, k, int(getattr(d, k)))
    for k in ["DELTAX", "DELTAY", "xobs", "yobs", "nu_0", "antenna_diameter", "pb_factor",
              "pb_cutoff"]:
        setattr(d, k, float(getattr(d, k)))
    return d


def test_fixtures_present():
    assert len(FIXTURES) >= 3, "golden fixtures of the reference kernels are missing"


@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: os.path.basename(p))
def test_oracle_matches_reference_kernels(path):
    g = load(path)
    orc = O.Oracle(g, TERMS + list(PRIOR_TERMS.values()))
    assert abs(orc.fg_scale - float(g.fg_scale)) <= 2e-6 * float(g.fg_scale)
    assert abs(orc.noise_cut - float(g.noise_cut)) <= 2e-6 * float(g.noise_cut)
    fin = np.isfinite(g.noise)
    assert np.array_equal(fin, np.isfinite(orc.noise))
    np.testing.assert_allclose(orc.noise[fin], g.noise[fin], rtol=5e-6)
    c0, _ = orc.chi2(orc.initial_image())
    assert abs(c0 - float(g.chi2_init)) <= 1e-5 * abs(float(g.chi2_init))
    c1, clipped = orc.chi2(g.img_rand.copy())
    assert abs(c1 - float(g.chi2_rand)) <= 1e-5 * abs(float(g.chi2_rand))
    np.testing.assert_array_equal(clipped, g.img_rand_clipped)
    res = orc.vr.reshape(-1, 2) * orc.weight[:, None]
    assert np.abs(res - g.res_rand).max() <= 1e-5 * np.abs(g.res_rand).max()
    grad = orc.dchi2(clipped)
    assert np.abs(grad - g.dchi2_rand).max() <= 1e-5 * np.abs(g.dchi2_rand[0]).max()
    for kind, t in PRIOR_TERMS.items():
        ti = 1 + list(PRIOR_TERMS).index(kind)
        v = orc.prior_value(ti, clipped)
        gv = float(g[f"prior{kind}_value"]) if isinstance(g, dict) else float(getattr(g, f"prior{kind}_value"))
        assert abs(v - gv) <= 1e-5 * max(abs(gv), 1e-30), (kind, v, gv)
        gg = getattr(g, f"prior{kind}_grad")
        og = orc.prior_grad(ti, clipped)
        assert np.abs(og - gg).max() <= 2e-5 * max(np.abs(gg).max(), 1e-30), kind


@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: os.path.basename(p))
def test_oracle_alpha_plane_matches_reference(path):
    g = load(path)
    orc = O.Oracle(g, TERMS)
    c, clipped = orc.chi2(g.img_alpha.copy(), flag_opt=1)
    assert abs(c - float(g.chi2_alpha)) <= 1e-5 * abs(float(g.chi2_alpha))
    np.testing.assert_array_equal(clipped, g.img_alpha_clipped)
    grad = orc.dchi2(clipped, flag_opt=1)
    mag = np.zeros_like(grad[1])
    for ch in range(len(g.freqs)):
        nud = np.float64(np.float32(g.freqs[ch]) / np.float32(g.nu_0))
        mag += np.abs(orc.dchi2_channel(ch) * clipped[0] * nud ** clipped[1] * orc.fg_scale * np.log(nud))
    assert np.abs(grad - g.dchi2_alpha).max() <= 1e-5 * mag.max()
