"""Error images (calculateErrors, src/functions.cu:4966-5041) on both DChi2
engines against an FP64 restatement of I_nu_0_Noise / alpha_Noise /
noise_reduction."""

import numpy as np
import pytest

import oracle as O
from gpuvmem_gb300 import synth

pytestmark = pytest.mark.gpu

TERMS = [(O.FI_CHI2, 1.0, 0, 0, 0.0, 0.0, 0.0)]


def error_images_fp64(data, orc, img_c):
    N, M = data.N, data.M
    x0, y0 = int(data.xobs), int(data.yobs)
    jj, ii = np.meshgrid(np.arange(M), np.arange(N))
    x = (jj - x0) * data.DELTAX * np.pi / 180.0
    y = (ii - y0) * data.DELTAY * np.pi / 180.0
    arc = np.sqrt(x * x + y * y)
    mask = orc.mask
    vr = orc.vr.reshape(-1, 2)
    E = np.zeros((2, N, M))
    for c in range(len(data.freqs)):
        o, e = data.chan_off[c], data.chan_off[c + 1]
        nu = float(data.freqs[c])
        lam = float(np.float32(2.99792458e8) / np.float32(nu))
        fwhm = data.pb_factor * lam / data.antenna_diameter
        atten = np.exp(-4.0 * np.log(2.0) * (arc / fwhm) ** 2) * (arc <= data.pb_cutoff)
        u, v = orc.uvw[o:e, 0], orc.uvw[o:e, 1]
        w = orc.weight[o:e].astype(np.float64)
        W = w.sum()
        nud = nu / float(data.nu_0)
        alpha = img_c[1].astype(np.float64)
        inu = img_c[0] * nud ** alpha
        ph = 2 * np.pi * (x[..., None] * u + y[..., None] * v)
        S = (w * (vr[o:e, 0] * np.cos(ph) - vr[o:e, 1] * np.sin(ph))).sum(-1)
        E[0] += np.where(mask, atten ** 2 * W * nud ** (2 * alpha), 0.0)
        s = atten * inu * W + S
        E[1] += np.where(mask & (s > 0), np.log(nud) ** 2 * atten * inu * s, 0.0)
    return np.where(E > 0, 1.0 / np.sqrt(np.where(E > 0, E, 1.0)), 0.0)


@pytest.mark.parametrize("engine", [1, 2])
def test_error_images_match_fp64(engine):
    import torch
    import gpuvmem_gb300 as gv
    cfg = synth.small_config(n=128, n_ant=10, n_times=48, nchan=3, seed=61)
    data = synth.generate(cfg)
    orc = O.Oracle(data, TERMS)
    prob = gv.Problem(data, TERMS, engine=engine)
    rng = np.random.default_rng(3)
    img = orc.initial_image()
    img[0] += ((rng.uniform(0, 1, img[0].shape) < 0.1) *
               np.abs(rng.normal(0, 3000.0, img[0].shape))).astype(np.float32)
    img[1] = rng.uniform(-1, 3, img[1].shape).astype(np.float32)
    _, img_c = orc.chi2(img.copy())
    ref = error_images_fp64(data, orc, img_c)
    got = prob.error_images(torch.from_numpy(img.copy()).cuda()).cpu().numpy()
    # compare the accumulated sums (1 / E^2): a pixel whose alpha sum s
    # lands near 0 may fall on either side of the s > 0 test
    for k in range(2):
        sg = np.where(got[k] > 0, 1.0 / np.where(got[k] > 0, got[k], 1.0) ** 2, 0.0)
        sr = np.where(ref[k] > 0, 1.0 / np.where(ref[k] > 0, ref[k], 1.0) ** 2, 0.0)
        assert np.abs(sg - sr).max() <= 1e-4 * np.abs(sr).max(), (k, np.abs(sg - sr).max())
        assert np.mean((got[k] == 0) != (ref[k] == 0)) < 1e-2
