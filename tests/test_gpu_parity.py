"""Parity of the CUDA path (through the C ABI) against the CPU oracle on the
same seeded inputs.  Tolerances are those of the reference parity gates:
chi2 within 1e-5 relative, gradients within 1e-5 * max|grad| per pixel,
images after a fixed number of iterations within 1e-4 of their peak."""

import numpy as np
import pytest

import oracle as O
from gpuvmem_gb300 import synth

pytestmark = pytest.mark.gpu

CHI2_RTOL = 1e-5
GRAD_TOL = 1e-5
IMG_TOL = 1e-4

ALL_PRIORS = [
    (O.FI_CHI2, 1.0, 0, 0, 0.0, 0.0, 0.0),
    (O.FI_ENTROPY, 0.01, 0, 0, 0.001, -1.0, 0.0),
    (O.FI_L1, 1e-3, 0, 0, 0.0, 0.0, 1e-12),
    (O.FI_TSV, 1e-4, 0, 0, 0.0, 0.0, 0.0),
    (O.FI_TV, 1e-4, 0, 0, 0.0, 0.0, 1e-12),
    (O.FI_LAPLACIAN, 1e-5, 0, 0, 0.0, 0.0, 0.0),
]


def _torch():
    import torch
    return torch


def make_pair(cfg, terms, **kw):
    import gpuvmem_gb300 as gv
    data = synth.generate(cfg)
    orc = O.Oracle(data, terms, **kw)
    prob = gv.Problem(data, [tuple(t) for t in terms], **kw)
    return data, orc, prob


def rand_image(orc, seed, alpha=False):
    rng = np.random.default_rng(seed)
    img = orc.initial_image()
    sparse = rng.uniform(0, 1, img[0].shape) < 0.2
    img[0] += (sparse * np.abs(rng.normal(0, 2000.0, img[0].shape))).astype(np.float32)
    if alpha:
        img[1] = rng.uniform(-1, 3, img[1].shape).astype(np.float32)
    return img


@pytest.fixture(scope="module")
def pair64():
    return make_pair(synth.small_config(n=64, nchan=2, seed=3), ALL_PRIORS)


@pytest.fixture(scope="module")
def pair128():
    return make_pair(synth.small_config(n=128, n_ant=10, n_times=60, nchan=1, seed=5),
                     ALL_PRIORS[:2])


def test_setup_matches_oracle(pair64):
    torch = _torch()
    data, orc, prob = pair64
    inf = prob.info
    assert abs(inf.fg_scale - orc.fg_scale) <= 1e-6 * orc.fg_scale
    assert abs(inf.noise_cut - orc.noise_cut) <= 1e-6 * orc.noise_cut
    assert inf.mask_pixels == int(orc.mask.sum())
    assert abs(inf.vis_noise - orc.vis_noise) <= 1e-6 * orc.vis_noise
    noise = prob.noise_image().cpu().numpy()
    fin = np.isfinite(orc.noise.reshape(noise.shape))
    assert np.array_equal(fin, np.isfinite(noise))
    np.testing.assert_allclose(noise[fin], orc.noise.reshape(noise.shape)[fin], rtol=2e-6)


@pytest.mark.parametrize("which", ["initial", "random"])
def test_chi2_and_clip(pair64, which):
    torch = _torch()
    data, orc, prob = pair64
    img = orc.initial_image() if which == "initial" else rand_image(orc, 7)
    ref, ref_img = orc.chi2(img.copy())
    d = torch.from_numpy(img.copy()).cuda()
    got = prob.chi2(d)
    assert abs(got - ref) <= CHI2_RTOL * abs(ref), (got, ref)
    # clip2IWNoise mutates the evaluated image
    np.testing.assert_array_equal(d.cpu().numpy(), ref_img)


def test_residuals_match(pair64):
    torch = _torch()
    data, orc, prob = pair64
    img = rand_image(orc, 11)
    orc.chi2(img.copy())
    prob.chi2(torch.from_numpy(img.copy()).cuda())
    got = prob.residuals()
    ref = orc.vr.reshape(-1, 2) * orc.weight[:, None]
    scale = np.abs(ref).max()
    assert np.abs(got - ref).max() <= 1e-5 * scale


@pytest.mark.parametrize("flag", [0, 1])
def test_dchi2(pair64, flag):
    torch = _torch()
    data, orc, prob = pair64
    img = rand_image(orc, 13, alpha=(flag == 1))
    _, img_c = orc.chi2(img.copy(), flag_opt=flag)
    ref = orc.dchi2(img_c, flag_opt=flag)
    d = torch.from_numpy(img.copy()).cuda()
    prob.chi2(d, flag)
    got = prob.dchi2(d, flag).cpu().numpy()
    plane = flag % 2
    scale = np.abs(ref[plane]).max()
    if plane == 1:
        # the alpha chain rule weights channels by log(nu/nu_0), which has
        # opposite signs either side of nu_0: the tolerance is taken
        # relative to the sum of the channel terms' magnitudes, not to
        # their (cancelling) sum
        mag = np.zeros_like(ref[1])
        for c in range(len(data.freqs)):
            nud = np.float64(np.float32(data.freqs[c]) / np.float32(data.nu_0))
            fac = img_c[0] * nud ** img_c[1] * orc.fg_scale * np.log(nud)
            mag += np.abs(orc.dchi2_channel(c) * fac)
        scale = mag.max()
    assert scale > 0
    err = np.abs(got - ref).max()
    assert err <= GRAD_TOL * scale, (err, scale)


def test_dchi2_channel_raw(pair64):
    torch = _torch()
    data, orc, prob = pair64
    img = rand_image(orc, 17)
    orc.chi2(img.copy())
    prob.chi2(torch.from_numpy(img.copy()).cuda())
    for c in range(len(data.freqs)):
        ref = orc.dchi2_channel(c)
        got = prob.dchi2_channel(c).cpu().numpy()
        assert np.abs(got - ref).max() <= GRAD_TOL * np.abs(ref).max()


@pytest.mark.parametrize("t", range(1, 6))
def test_prior_value_and_gradient(pair64, t):
    torch = _torch()
    data, orc, prob = pair64
    img = rand_image(orc, 19 + t)
    _, img = orc.chi2(img.copy())  # priors see the clipped image
    d = torch.from_numpy(img.copy()).cuda()
    ref_v = orc.prior_value(t, img)
    got_v = prob.prior_value(t, d)
    assert abs(got_v - ref_v) <= 1e-5 * max(abs(ref_v), 1e-30), (got_v, ref_v)
    ref_g = orc.prior_grad(t, img)
    got_g = prob.prior_gradient(t, d).cpu().numpy()
    add = 0 if ALL_PRIORS[t][0] == O.FI_TV else ALL_PRIORS[t][3]
    scale = max(np.abs(ref_g).max(), 1e-30)
    assert np.abs(got_g[add] - ref_g).max() <= 2e-5 * scale


def _extra_priors(n):
    """GEntropy and GL1Norm over a seeded prior image (factor 2 and 1), and
    Quadratic; the prior stays below the image so every term is positive."""
    rng = np.random.default_rng(77)
    prior = rng.uniform(1e-4, 9e-4, (n, n)).astype(np.float32)
    return [(O.FI_CHI2, 1.0, 0, 0, 0.0, 0.0, 0.0),
            (O.FI_GENTROPY, 0.01, 0, 0, 0.0, -1.0, 0.0, prior, 2.0, 0.0),
            (O.FI_GL1, 1e-3, 0, 0, 0.0, 0.0, 1e-12, prior, 1.0, 1e-12),
            (O.FI_QUADRATIC, 1e-5, 0, 0, 0.0, 0.0, 0.0)]


@pytest.fixture(scope="module")
def pair64_extra():
    return make_pair(synth.small_config(n=64, nchan=2, seed=3), _extra_priors(64))


@pytest.mark.parametrize("t", range(1, 4))
def test_extra_prior_value_and_gradient(pair64_extra, t):
    """GEntropy (src/gentropy.cu), GL1Norm (src/gl1norm.cu) and Quadratic
    (src/quadraticpenalization.cu) against the oracle."""
    torch = _torch()
    data, orc, prob = pair64_extra
    img = rand_image(orc, 41 + t)
    _, img = orc.chi2(img.copy())
    d = torch.from_numpy(img.copy()).cuda()
    ref_v = orc.prior_value(t, img)
    got_v = prob.prior_value(t, d)
    assert ref_v > 0
    assert abs(got_v - ref_v) <= 1e-5 * ref_v, (got_v, ref_v)
    ref_g = orc.prior_grad(t, img)
    got_g = prob.prior_gradient(t, d).cpu().numpy()
    scale = np.abs(ref_g).max()
    assert scale > 0
    assert np.abs(got_g[0] - ref_g).max() <= 2e-5 * scale


def test_extra_priors_objective(pair64_extra):
    """The whole objective with the three extra priors active (iteration 1)."""
    torch = _torch()
    data, orc, prob = pair64_extra
    img = rand_image(orc, 51)
    d = torch.from_numpy(img.copy()).cuda()
    orc.state.iteration = 1
    f_ref, _ = orc.calc_function(img.copy())
    prob.set_iteration(1)
    f_got, _ = prob.objective(d)
    prob.set_iteration(0)
    orc.state.iteration = 0
    assert abs(f_got - f_ref) <= CHI2_RTOL * abs(f_ref), (f_got, f_ref)


def test_objective_and_gradient_iteration_gating(pair64):
    torch = _torch()
    data, orc, prob = pair64
    img = rand_image(orc, 29)
    d = torch.from_numpy(img.copy()).cuda()
    orc.state.iteration = 0
    f0, img_c = orc.calc_function(img.copy())
    g0, _ = prob.objective(d)
    assert abs(g0 - f0) <= CHI2_RTOL * abs(f0)
    # calcGradient sees the image calcFunction clipped in place
    ref_xi = orc.calc_gradient(img_c, 1)
    got_xi = prob.gradient(d, 1).cpu().numpy()
    assert np.abs(got_xi - ref_xi).max() <= GRAD_TOL * np.abs(ref_xi).max()
    # after a gradient call with iter > 0 the priors enter the objective
    f1, _ = orc.calc_function(img.copy())
    g1, fi = prob.objective(d)
    assert f1 != f0
    assert abs(g1 - f1) <= CHI2_RTOL * abs(f1)


def test_chi2_larger_image(pair128):
    torch = _torch()
    data, orc, prob = pair128
    img = rand_image(orc, 31)
    ref, _ = orc.chi2(img.copy())
    d = torch.from_numpy(img.copy()).cuda()
    assert abs(prob.chi2(d) - ref) <= CHI2_RTOL * abs(ref)
    ref_g = orc.dchi2(orc.chi2(img.copy())[1])
    got_g = prob.dchi2(d).cpu().numpy()
    assert np.abs(got_g - ref_g).max() <= GRAD_TOL * np.abs(ref_g[0]).max()


def test_dirty_image(pair64):
    torch = _torch()
    data, orc, prob = pair64
    got = prob.dirty_image().cpu().numpy()
    orc.chi2(orc.initial_image())  # vis_mod zeroes out-of-grid weights
    x0, y0 = int(data.xobs), int(data.yobs)
    jj, ii = np.meshgrid(np.arange(data.M), np.arange(data.N))
    x = (jj - x0) * data.DELTAX * np.pi / 180.0
    y = (ii - y0) * data.DELTAY * np.pi / 180.0
    zm1 = np.sqrt(1.0 - x * x - y * y) - 1.0
    ref = np.zeros((data.N, data.M))
    for c in range(len(data.freqs)):
        o, e = data.chan_off[c], data.chan_off[c + 1]
        u, v, w = orc.uvw[o:e, 0], orc.uvw[o:e, 1], orc.uvw[o:e, 2]
        wt, vo = orc.weight[o:e].astype(np.float64), orc.vo[o:e].astype(np.float64)
        ph = 2 * np.pi * (x[..., None] * u + y[..., None] * v + zm1[..., None] * w)
        ref += (wt * (vo[:, 0] * np.cos(ph) + vo[:, 1] * np.sin(ph))).sum(-1)
    assert np.abs(got - ref).max() <= 1e-5 * np.abs(ref).max()


def test_psf_image(pair64):
    """PSF = the adjoint applied to the weights (Vr := 1): sum_k w_k cos(phase)."""
    data, orc, prob = pair64
    got = prob.psf_image().cpu().numpy()
    orc.chi2(orc.initial_image())
    x0, y0 = int(data.xobs), int(data.yobs)
    jj, ii = np.meshgrid(np.arange(data.M), np.arange(data.N))
    x = (jj - x0) * data.DELTAX * np.pi / 180.0
    y = (ii - y0) * data.DELTAY * np.pi / 180.0
    zm1 = np.sqrt(1.0 - x * x - y * y) - 1.0
    ref = np.zeros((data.N, data.M))
    for c in range(len(data.freqs)):
        o, e = data.chan_off[c], data.chan_off[c + 1]
        u, v, w = orc.uvw[o:e, 0], orc.uvw[o:e, 1], orc.uvw[o:e, 2]
        wt = orc.weight[o:e].astype(np.float64)
        ph = 2 * np.pi * (x[..., None] * u + y[..., None] * v + zm1[..., None] * w)
        ref += (wt * np.cos(ph)).sum(-1)
    assert np.abs(got - ref).max() <= 1e-5 * np.abs(ref).max()
    assert abs(ref[y0, x0] - orc.weight.astype(np.float64).sum()) <= 1e-9 * ref[y0, x0]


@pytest.mark.parametrize("method", ["frprmn", "lbfgs"])
def test_optimizer_trajectory(method):
    """Image after a fixed number of iterations.  Brent's minimiser works on
    float objective values, so each line search fixes its step only to about
    sqrt(FLT_EPSILON) relative; two implementations whose objectives differ
    in the last float bits separate at that rate per iteration (measured:
    5e-6 of the peak after 2 iterations, 1.6e-4 after 4).  The image gate is
    therefore checked at 2 iterations and the objective after 6."""
    torch = _torch()
    data, orc, prob = make_pair(synth.small_config(n=64, nchan=1, seed=9), ALL_PRIORS[:2])
    iters = 2
    img0 = orc.initial_image()
    ref_img, ref_rep = orc.optimize(img0.copy(), method, iterations=iters, K=5)
    d = torch.from_numpy(img0.copy()).cuda()
    rep = prob.optimize(d, "CG-FRPRMN" if method == "frprmn" else "CG-LBFGS", iterations=iters, K=5)
    got = d.cpu().numpy()
    assert rep.iterations == ref_rep.iterations
    peak = np.abs(ref_img[0]).max()
    assert np.abs(got - ref_img).max() <= IMG_TOL * peak, (np.abs(got - ref_img).max(), peak)
    assert abs(rep.f_final - ref_rep.f_final) <= 1e-4 * abs(ref_rep.f_final)


@pytest.mark.parametrize("method", ["frprmn", "lbfgs"])
def test_optimizer_objective_after_6(method):
    torch = _torch()
    data, orc, prob = make_pair(synth.small_config(n=64, nchan=1, seed=9), ALL_PRIORS[:2])
    img0 = orc.initial_image()
    _, ref_rep = orc.optimize(img0.copy(), method, iterations=6, K=5)
    d = torch.from_numpy(img0.copy()).cuda()
    rep = prob.optimize(d, "CG-FRPRMN" if method == "frprmn" else "CG-LBFGS", iterations=6, K=5)
    assert rep.iterations == ref_rep.iterations
    assert abs(rep.f_final - ref_rep.f_final) <= 1e-3 * abs(ref_rep.f_final)
