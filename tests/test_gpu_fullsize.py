"""Parity at the benchmark configurations' real sizes, through the C ABI.

  plain MEM 256^2, 1 channel, 104,400 visibilities: set-up, chi2, the whole
      gradient (tensor-core engine), prior values and gradients, the full
      objective and two frprmn iterations, against the FP64 oracle in full
      and against the reference's own kernels run live;
  plain MEM 2048^2, 8 channels, 35.28M visibilities (Briggs): set-up and
      chi2 in full; the gradient at sampled pixels against the FP64 oracle's
      direct sum over every visibility of every channel, and over a band of
      16 rows against the reference's own DChi2 kernels;
  batched MFS 1024^2, 64 channels (flagged): the I_nu0 and alpha planes of
      the gradient at sampled pixels against the FP64 oracle.

Gates: chi2 within 1e-5 relative; gradients within 1e-5 * max|grad| per
pixel; images after a fixed iteration count within 1e-4 of their peak.  Each
test prints the errors of both sides against the FP64 oracle.
"""

import numpy as np
import pytest

import oracle as O
import refrun
from gpuvmem_gb300 import synth

pytestmark = pytest.mark.gpu

CHI2_RTOL = 1e-5
GRAD_TOL = 1e-5
IMG_TOL = 1e-4
TERMS = [(O.FI_CHI2, 1.0, 0, 0, 0.0, 0.0, 0.0),
         (O.FI_ENTROPY, 0.01, 0, 0, 0.001, -1.0, 0.0),
         (O.FI_TSV, 1e-4, 0, 0, 0.0, 0.0, 0.0)]


def sparse_image(orc, seed, density=0.05, alpha=False):
    rng = np.random.default_rng(seed)
    img = orc.initial_image()
    on = rng.uniform(0, 1, img[0].shape) < density
    img[0] += (on * np.abs(rng.normal(0, 2000.0, img[0].shape))).astype(np.float32)
    if alpha:
        img[1] = rng.uniform(-1, 3, img[1].shape).astype(np.float32)
    return img


def attenuation(data, i, j, freq):
    return O.lib().or_attenuation(int(i), int(j), data.xobs, data.yobs, data.DELTAX, data.DELTAY,
                                  float(freq), data.antenna_diameter, data.pb_factor,
                                  data.pb_cutoff, data.primary_beam)


def oracle_grad_pixels(orc, data, img_c, pix, flag):
    """The FP64 oracle's gradient of chi2 at pixels `pix` (plane flag % 2):
    DChi2's direct sum over every visibility of every channel
    (src/functions.cu:3698-3791) with the DChi2_total_I_nu_0 / _alpha chain
    rule (:3968-4024).  Also returns, per pixel, the sum of the channel
    terms' magnitudes (the alpha chain rule's log(nu/nu_0) changes sign
    across nu_0, so its channel terms cancel)."""
    N = data.N
    MN = data.M * N
    i0 = img_c[0].reshape(-1)[pix].astype(np.float64)
    al = img_c[1].reshape(-1)[pix].astype(np.float64)
    g = np.zeros(len(pix))
    mag = np.zeros(len(pix))
    for c in range(len(data.freqs)):
        if data.chan_off[c + 1] == data.chan_off[c]:
            continue
        s = orc.dchi2_pixels(c, pix)
        a = np.array([attenuation(data, q // N, q % N, orc.freqs[c]) for q in pix])
        tmp = -s * np.float64(orc.fg_scale) * a
        nudiv = np.float64(np.float32(orc.freqs[c]) / np.float32(data.nu_0))
        pw = nudiv ** al
        if flag % 2 == 0:
            term = tmp * pw
        else:
            term = np.where(i0 > 0.0, tmp * (i0 * pw * np.float64(orc.fg_scale) * np.log(nudiv)),
                            0.0)
        g += term
        mag += np.abs(term)
    assert MN > 0
    return g, mag


def sample_pixels(mask, rng, n, extra=()):
    idx = np.flatnonzero(mask.reshape(-1))
    pick = rng.choice(idx, size=min(n, idx.size), replace=False)
    return np.unique(np.concatenate([pick, np.asarray(extra, dtype=np.int64)])).astype(np.int64)


# ---- plain MEM 256^2 -------------------------------------------------------

@pytest.fixture(scope="module")
def plain256():
    import gpuvmem_gb300 as gv
    data = synth.generate(synth.CONFIG0)
    orc = O.Oracle(data, TERMS)
    prob = gv.Problem(data, [tuple(t) for t in TERMS])
    yield data, orc, prob
    prob.close()


def test_plain256_setup(plain256):
    data, orc, prob = plain256
    inf = prob.info
    assert data.nvis == 104400
    assert abs(inf.fg_scale - orc.fg_scale) <= 1e-6 * orc.fg_scale
    assert abs(inf.noise_cut - orc.noise_cut) <= 1e-6 * orc.noise_cut
    assert abs(inf.vis_noise - orc.vis_noise) <= 1e-6 * orc.vis_noise
    assert inf.mask_pixels == int(orc.mask.sum())


def test_plain256_chi2_gradient_full(plain256):
    import torch
    data, orc, prob = plain256
    assert prob.info.dchi2_engine == 2
    img = sparse_image(orc, 101)
    c_orc, img_c = orc.chi2(img.copy())
    d = torch.from_numpy(img.copy()).cuda()
    c_ours = prob.chi2(d)
    np.testing.assert_array_equal(d.cpu().numpy(), img_c)
    g_orc = orc.dchi2(img_c)
    g_ours = prob.dchi2(d).cpu().numpy()
    scale = np.abs(g_orc[0]).max()
    e_c = abs(c_ours - c_orc) / abs(c_orc)
    e_g = np.abs(g_ours - g_orc).max() / scale
    print(f"\nplain 256^2: chi2 rel err vs oracle {e_c:.2e}; gradient {e_g:.2e} of max|grad|")
    assert e_c <= CHI2_RTOL
    assert e_g <= GRAD_TOL


@pytest.mark.skipif(not refrun.available(), reason="reference kernels cubin not built")
def test_plain256_vs_reference_kernels(plain256):
    import torch
    data, orc, prob = plain256
    ref = refrun.RefHarness(data)
    try:
        assert abs(prob.info.fg_scale - ref.fg_scale) <= 2e-6 * ref.fg_scale
        img = sparse_image(orc, 103)
        c_ref, img_ref = ref.chi2(img)
        c_orc, img_orc = orc.chi2(img.copy())
        d = torch.from_numpy(img.copy()).cuda()
        c_ours = prob.chi2(d)
        np.testing.assert_array_equal(d.cpu().numpy(), img_ref)
        g_ref = ref.dchi2(img_ref)
        g_orc = orc.dchi2(img_orc)
        g_ours = prob.dchi2(d).cpu().numpy()
        scale = np.abs(g_orc[0]).max()
        e = {"chi2 ours-ref": abs(c_ours - c_ref) / abs(c_ref),
             "chi2 ref-oracle": abs(c_ref - c_orc) / abs(c_orc),
             "chi2 ours-oracle": abs(c_ours - c_orc) / abs(c_orc),
             "grad ours-ref": np.abs(g_ours - g_ref).max() / scale,
             "grad ref-oracle": np.abs(g_ref - g_orc).max() / scale,
             "grad ours-oracle": np.abs(g_ours - g_orc).max() / scale}
        # priors: value and lambda * gradient of the reference's kernels
        for kind, lam in ((1, 0.01), (2, 1e-4)):
            v_ref, gr_ref = ref.prior(kind, lam, img_ref)
            ti = 1 if kind == 1 else 2
            v_orc = orc.prior_value(ti, img_orc)
            v_ours = prob.prior_value(ti, d)
            gp = prob.prior_gradient(ti, d).cpu().numpy()[0]
            gp_orc = orc.prior_grad(ti, img_orc)  # lambda * gradient
            e[f"prior {kind} value ours-ref"] = abs(v_ours - v_ref) / abs(v_ref)
            e[f"prior {kind} value ours-oracle"] = abs(v_ours - v_orc) / abs(v_orc)
            e[f"prior {kind} grad ours-ref"] = np.abs(gp - gr_ref).max() / np.abs(gp_orc).max()
            e[f"prior {kind} grad ours-oracle"] = np.abs(gp - gp_orc).max() / np.abs(gp_orc).max()
        print("\n" + "; ".join(f"{k} {v:.2e}" for k, v in e.items()))
        assert e["chi2 ours-ref"] <= CHI2_RTOL
        assert e["grad ours-ref"] <= GRAD_TOL
        assert e["grad ours-oracle"] <= GRAD_TOL
        for kind in (1, 2):
            assert e[f"prior {kind} value ours-ref"] <= CHI2_RTOL
            assert e[f"prior {kind} grad ours-ref"] <= GRAD_TOL
            assert e[f"prior {kind} grad ours-oracle"] <= GRAD_TOL
    finally:
        ref.close()


def test_plain256_objective_and_frprmn(plain256):
    """The whole objective with its priors active (iteration > 0), its
    gradient, and the image after one (gated) and two (printed) frprmn
    iterations from the initial image."""
    import torch
    data, orc, prob = plain256
    img = sparse_image(orc, 105)
    orc.state.iteration = 1
    f_orc, img_c = orc.calc_function(img.copy())
    xi_orc = orc.calc_gradient(img_c, 1)
    d = torch.from_numpy(img.copy()).cuda()
    prob.set_iteration(1)
    f_ours, _ = prob.objective(d)
    xi = prob.gradient(d, 1).cpu().numpy()
    e_f = abs(f_ours - f_orc) / abs(f_orc)
    e_g = np.abs(xi - xi_orc).max() / np.abs(xi_orc).max()
    prob.set_iteration(0)
    x0 = orc.initial_image()
    e_i = []
    for iters in (1, 2):
        x_orc, rep_orc = orc.optimize(x0.copy(), "frprmn", iterations=iters)
        dx = torch.from_numpy(x0.copy()).cuda()
        prob.optimize(dx, "CG-FRPRMN", iterations=iters)
        x_ours = dx.cpu().numpy()
        e_i.append(np.abs(x_ours - x_orc).max() / np.abs(x_orc).max())
    print(f"\nplain 256^2: objective rel err {e_f:.2e}; gradient {e_g:.2e} of max; "
          f"image after 1 / 2 frprmn iterations {e_i[0]:.2e} / {e_i[1]:.2e} of its peak")
    assert e_f <= CHI2_RTOL
    assert e_g <= GRAD_TOL
    # Brent's float line search fixes each step to about sqrt(FLT_EPSILON):
    # objectives that differ in the last bits separate at that rate per
    # iteration, so the image gate is taken after the first iteration
    assert e_i[0] <= IMG_TOL


# ---- plain MEM 2048^2, 8 channels, 35.28M visibilities ---------------------

@pytest.fixture(scope="module")
def plain2048():
    import gpuvmem_gb300 as gv
    data = synth.generate(synth.CONFIG1, device="cuda")
    orc = O.Oracle(data, TERMS)
    prob = gv.Problem(data, [tuple(t) for t in TERMS])
    yield data, orc, prob
    prob.close()


def test_plain2048_setup_and_chi2(plain2048):
    import torch
    data, orc, prob = plain2048
    inf = prob.info
    assert data.nvis == 35280000
    assert abs(inf.fg_scale - orc.fg_scale) <= 1e-6 * orc.fg_scale
    assert abs(inf.noise_cut - orc.noise_cut) <= 1e-6 * orc.noise_cut
    assert inf.mask_pixels == int(orc.mask.sum())
    img = sparse_image(orc, 201, density=0.01)
    c_orc, img_c = orc.chi2(img.copy())
    d = torch.from_numpy(img.copy()).cuda()
    c_ours = prob.chi2(d)
    np.testing.assert_array_equal(d.cpu().numpy(), img_c)
    e = abs(c_ours - c_orc) / abs(c_orc)
    print(f"\nplain 2048^2: chi2 rel err vs oracle {e:.2e}")
    assert e <= CHI2_RTOL


def test_plain2048_gradient_sampled(plain2048):
    """DChi2 (tcgen05 engine, every visibility of every channel) at 256
    random mask pixels plus the pixel of largest |gradient|, against the
    FP64 oracle's direct sum over all 35.28M visibilities; and over a band
    of 16 rows through that pixel against the reference's own kernels."""
    import torch
    data, orc, prob = plain2048
    assert prob.info.dchi2_engine == 2
    img = sparse_image(orc, 203, density=0.01)
    _, img_c = orc.chi2(img.copy())
    d = torch.from_numpy(img.copy()).cuda()
    prob.chi2(d)
    g_ours = prob.dchi2(d).cpu().numpy()
    qmax = int(np.abs(g_ours[0]).argmax())
    rng = np.random.default_rng(7)
    pix = sample_pixels(orc.mask, rng, 256, extra=[qmax])
    g_orc, _ = oracle_grad_pixels(orc, data, img_c, pix, 0)
    scale = np.abs(g_orc).max()
    assert scale >= 0.99 * np.abs(g_ours[0]).max()
    got = g_ours[0].reshape(-1)[pix]
    e_ours = np.abs(got - g_orc).max() / scale
    msg = f"\nplain 2048^2: gradient ours-oracle {e_ours:.2e} of max|grad| at {pix.size} pixels"
    if refrun.available():
        ref = refrun.RefHarness(data)
        try:
            _, img_ref = ref.chi2(img)
            np.testing.assert_array_equal(img_ref, img_c)
            row = qmax // data.N
            i0 = min(max(0, row // 16 * 16), data.N - 16)
            band = ref.dchi2_band(img_ref, i0, 16)[0]
            ours_band = g_ours[0, i0:i0 + 16]
            diff = np.abs(ours_band - band).reshape(-1)
            e_band = diff.max() / scale
            # the oracle decides at the 32 pixels where ours and the
            # reference disagree most, plus 32 random ones of the band
            inband = np.arange(i0 * data.N, (i0 + 16) * data.N)
            worst = np.argsort(diff)[-32:] + i0 * data.N
            bp = sample_pixels(orc.mask.reshape(-1)[inband], rng, 32) + i0 * data.N
            bp = np.unique(np.concatenate([bp, worst, [qmax]])).astype(np.int64)
            g_orc_b, _ = oracle_grad_pixels(orc, data, img_c, bp, 0)
            e_ref_orc = np.abs(band.reshape(-1)[bp - i0 * data.N] - g_orc_b).max() / scale
            e_ours_orc_b = np.abs(g_ours[0].reshape(-1)[bp] - g_orc_b).max() / scale
            msg += (f"; rows {i0}-{i0 + 15} ({band.size} pixels): ours-ref max {e_band:.2e}; at "
                    f"{bp.size} pixels incl. the 32 largest disagreements: ref-oracle "
                    f"{e_ref_orc:.2e}, ours-oracle {e_ours_orc_b:.2e}")
            # the reference's FP32 running sum over 4.41M visibilities per
            # channel is itself off the FP64 value by more than the gate:
            # where the two disagree, ours is the one within the gate
            assert e_ours_orc_b <= GRAD_TOL
            assert e_band <= e_ref_orc + GRAD_TOL
        finally:
            ref.close()
    print(msg)
    assert e_ours <= GRAD_TOL


def test_plain2048_objective_with_priors(plain2048):
    import torch
    data, orc, prob = plain2048
    img = sparse_image(orc, 205, density=0.01)
    orc.state.iteration = 1
    f_orc, _ = orc.calc_function(img.copy())
    fi_orc = list(orc.state.last_fi)[:len(TERMS)]
    prob.set_iteration(1)
    d = torch.from_numpy(img.copy()).cuda()
    f_ours, fi = prob.objective(d)
    prob.set_iteration(0)
    e = abs(f_ours - f_orc) / abs(f_orc)
    print(f"\nplain 2048^2 objective: rel err {e:.2e}; terms ours {fi} oracle {fi_orc}")
    assert e <= CHI2_RTOL
    for a, b in zip(fi, fi_orc):
        assert abs(a - b) <= CHI2_RTOL * max(abs(b), 1e-30)


# ---- batched MFS 1024^2, 64 channels ---------------------------------------

@pytest.fixture(scope="module")
def mfs1024():
    import gpuvmem_gb300 as gv
    data = synth.generate(synth.CONFIG2, device="cuda")
    orc = O.Oracle(data, TERMS[:2])
    prob = gv.Problem(data, [tuple(t) for t in TERMS[:2]])
    yield data, orc, prob
    prob.close()


@pytest.mark.parametrize("flag", [0, 1])
def test_mfs1024_planes_sampled(mfs1024, flag):
    """Both MFS planes (flag 0: I_nu0, flag 1: alpha) over 64 channels of
    uneven visibility counts, at 192 sampled mask pixels."""
    import torch
    data, orc, prob = mfs1024
    img = sparse_image(orc, 301 + flag, density=0.05, alpha=True)
    c_orc, img_c = orc.chi2(img.copy(), flag_opt=flag)
    d = torch.from_numpy(img.copy()).cuda()
    c_ours = prob.chi2(d, flag)
    np.testing.assert_array_equal(d.cpu().numpy(), img_c)
    g_ours = prob.dchi2(d, flag).cpu().numpy()
    plane = flag % 2
    qmax = int(np.abs(g_ours[plane]).argmax())
    rng = np.random.default_rng(11 + flag)
    pix = sample_pixels(orc.mask, rng, 192, extra=[qmax])
    g_orc, mag = oracle_grad_pixels(orc, data, img_c, pix, flag)
    scale = mag.max() if plane == 1 else np.abs(g_orc).max()
    got = g_ours[plane].reshape(-1)[pix]
    e_c = abs(c_ours - c_orc) / abs(c_orc)
    e_g = np.abs(got - g_orc).max() / scale
    print(f"\nMFS 1024^2 x 64 channels flag {flag}: {data.nvis} visibilities; chi2 rel err "
          f"{e_c:.2e}; gradient plane {plane} {e_g:.2e} of max at {pix.size} pixels")
    assert e_c <= CHI2_RTOL
    assert e_g <= GRAD_TOL


# ---- calculateNoiseAndBeam on the GPU ---------------------------------------

@pytest.mark.parametrize("which", ["plain256", "plain2048"])
def test_noise_and_beam_on_gpu(which, request):
    """calculateNoiseAndBeam (src/functions.cu:1700-1814): the FP32 weight
    sum (the reference's uncompensated sequential sum) bit for bit, the beam
    moments and the visibility noise against the oracle."""
    data, orc, prob = request.getfixturevalue(which)
    inf = prob.info
    assert np.float32(inf.sum_weights).tobytes() == np.float32(orc.sum_weights).tobytes(), \
        (inf.sum_weights, orc.sum_weights)
    for a, b in ((inf.beam_bmaj_deg, orc.bmaj), (inf.beam_bmin_deg, orc.bmin),
                 (inf.beam_bpa_deg, orc.bpa)):
        assert abs(a - b) <= 1e-9 * max(abs(b), 1e-30), (a, b)
    assert np.float32(inf.vis_noise).tobytes() == np.float32(orc.vis_noise).tobytes()
