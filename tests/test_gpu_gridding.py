"""Convolutional gridding on the GPU (gv_grid_visibilities) against the
reference's own do_gridding (golden vectors, bit for bit), and the objective
path on gridded data with the gridding correction function (apply_GCF and
the GCF variant of DChi2) against the FP64 oracle with the same GCF."""

import glob
import math
import os

import numpy as np
import pytest

import oracle as O
from gpuvmem_gb300 import synth

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = sorted(glob.glob(os.path.join(HERE, "golden", "grid_*.npz")))
CHI2_RTOL = 1e-5
GRAD_TOL = 1e-5


@pytest.mark.parametrize("path", CASES, ids=lambda p: os.path.basename(p)[:-4])
def test_grid_matches_reference(path):
    import gpuvmem_gb300 as gv
    z = np.load(path)
    off, uvw, vo, w = gv.grid_visibilities(z["kernel"], tuple(z["support"]), int(z["M"]),
                                           int(z["N"]), float(z["deltax_deg"]),
                                           float(z["deltay_deg"]), z["freqs"], z["chan_off"],
                                           z["uvw_m"], z["vo"], z["weight"])
    np.testing.assert_array_equal(np.diff(off), z["counts"])
    np.testing.assert_array_equal(uvw, z["out_uvw"])
    np.testing.assert_array_equal(vo.view(np.uint32), z["out_vo"].view(np.uint32))
    np.testing.assert_array_equal(w.view(np.uint32), z["out_weight"].view(np.uint32))


def test_pillbox_cells_at_configuration0_size():
    """PillBox (1 x 1) at 256 x 256 with 104,400 visibilities: one output
    per distinct in-grid cell of the visibilities and their Hermitian copies,
    with the effective weight (sum w k)^2 / sum w k^2 = sum w of the cell
    (k = 1)."""
    import gpuvmem_gb300 as gv
    d = synth.generate(synth.CONFIG0)
    g, gcf = gv.grid(d, "PillBox2D")
    assert gcf is not None and np.all(gcf == 1.0)
    lam = np.float64(np.float32(np.float32(2.99792458e8) / np.float32(d.freqs[0])))
    du = 1.0 / (d.M * (math.pi / 180.0 * d.DELTAX))
    dv = 1.0 / (d.N * (math.pi / 180.0 * d.DELTAY))
    u = np.concatenate([d.uvw_m[:, 0], -d.uvw_m[:, 0]]) / lam
    v = np.concatenate([d.uvw_m[:, 1], -d.uvw_m[:, 1]]) / lam
    j = np.trunc((u / du + d.N // 2) + 0.5).astype(np.int64)
    k = np.trunc((v / dv + d.M // 2) + 0.5).astype(np.int64)
    ok = (j >= 0) & (j < d.N) & (k >= 0) & (k < d.M)
    cells = (d.N * k + j)[ok]
    ww = np.concatenate([d.weight, d.weight]).astype(np.float64)[ok]
    uniq = np.unique(cells)
    assert g.nvis == len(uniq) and g.nvis > 1000
    s1 = np.bincount(cells, ww, d.M * d.N)[uniq]
    np.testing.assert_allclose(g.weight, s1, rtol=1e-4)
    assert np.all(g.uvw_m[:, 2] == 0.0)


TERMS = [(O.FI_CHI2, 1.0, 0, 0, 0.0, 0.0, 0.0), (O.FI_ENTROPY, 0.01, 0, 0, 0.001, -1.0, 0.0)]


def _rand_image(orc, seed):
    rng = np.random.default_rng(seed)
    img = orc.initial_image()
    sparse = rng.uniform(0, 1, img[0].shape) < 0.2
    img[0] += (sparse * np.abs(rng.normal(0, 2000.0, img[0].shape))).astype(np.float32)
    return img


@pytest.mark.parametrize("kernel,engine", [("PSWF", 1), ("PSWF", 2), ("Gaussian2D", 2),
                                           ("PillBox2D", 2)])
def test_gridded_objective_with_gcf(kernel, engine):
    import torch
    import gpuvmem_gb300 as gv
    d = synth.generate(synth.small_config(n=128, n_ant=10, n_times=60, nchan=2, seed=9))
    g, gcf = gv.grid(d, kernel)
    assert g.nvis > 100
    orc = O.Oracle(g, TERMS, gcf=gcf)
    prob = gv.Problem(g, TERMS, engine=engine, gcf=gcf)
    assert prob.info.dchi2_engine == engine
    img = _rand_image(orc, 21)
    ref, img_c = orc.chi2(img.copy())
    dimg = torch.from_numpy(img.copy()).cuda()
    got = prob.chi2(dimg)
    assert abs(got - ref) <= CHI2_RTOL * abs(ref), (got, ref)
    ref_g = orc.dchi2(img_c)
    got_g = prob.dchi2(dimg).cpu().numpy()
    scale = np.abs(ref_g[0]).max()
    assert scale > 0
    assert np.abs(got_g - ref_g).max() <= GRAD_TOL * scale
    # without the GCF the result differs wherever the GCF is not 1
    if not np.all(gcf == 1.0):
        plain = gv.Problem(g, TERMS, engine=engine)
        d2 = torch.from_numpy(img.copy()).cuda()
        assert abs(plain.chi2(d2) - got) > 10 * CHI2_RTOL * abs(ref)
