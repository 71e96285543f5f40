"""The two-image MFS fit (I_nu0 and spectral index alpha) with MFS::run's
flag sequence 0, 1, 2, 3 (src/mfs.cu:999-1008), against the FP64 oracle's
optimiser on the same start.

Each stage starts both solvers from the same image (the oracle's previous
stage).  The I_nu0 stages (flags 0 and 2) are well conditioned: the images
agree within 1e-4 of the plane's peak.  Along alpha (flags 1 and 3) the
objective is flat to a few float ulps -- the alpha gradient carries the
factor fg_scale (DChi2_total_alpha, src/functions.cu:3968-3998) and is
about 1e-6 here while f is about 1e7 -- so which point a float line search
settles on is decided by rounding (the reference's FP32 chi2 has more
rounding noise still).  There the test checks what is well posed: the I_nu0
plane is untouched.  The sequence run in one call equals the four stages run
one after another."""

import dataclasses

import numpy as np
import pytest

import oracle as O
from gpuvmem_gb300 import synth

pytestmark = pytest.mark.gpu

IMG_TOL = 1e-4
TERMS = [(O.FI_CHI2, 1.0, 0, 0, 0.0, 0.0, 0.0), (O.FI_ENTROPY, 0.01, 0, 0, 0.001, -1.0, 0.0)]


def _setup():
    import gpuvmem_gb300 as gv
    cfg = dataclasses.replace(synth.small_config(n=64, n_ant=10, n_times=40, nchan=4, seed=31),
                              freqs_hz=list(np.linspace(85e9, 115e9, 4)), alpha_range=(-1.0, 3.0))
    data = synth.generate(cfg)
    orc = O.Oracle(data, TERMS)
    prob = gv.Problem(data, [tuple(t) for t in TERMS])
    rng = np.random.default_rng(5)
    img = orc.initial_image()
    on = rng.uniform(0, 1, img[0].shape) < 0.05
    img[0] += (on * np.abs(rng.normal(0, 2000.0, img[0].shape))).astype(np.float32)
    img[1] = (on * rng.uniform(-1, 3, img[0].shape)).astype(np.float32)
    return data, orc, prob, img


@pytest.mark.parametrize("method", ["CG-FRPRMN", "CG-LBFGS"])
def test_mfs_four_flag_stages(method):
    import torch
    data, orc, prob, img = _setup()
    om = "frprmn" if method == "CG-FRPRMN" else "lbfgs"
    notes = []
    for flag in (0, 1, 2, 3):
        x_orc, r_orc = orc.optimize(img.copy(), om, iterations=2, flag_opt=flag)
        d = torch.from_numpy(img.copy()).cuda()
        rep = prob.mfs_run(d, method, iterations=2, flags=(flag,))[0]
        x = d.cpu().numpy()
        e0 = np.abs(x[0] - x_orc[0]).max() / np.abs(x_orc[0]).max()
        e1 = np.abs(x[1] - x_orc[1]).max() / max(np.abs(x_orc[1]).max(), 1e-30)
        notes.append(f"flag {flag}: I_nu0 {e0:.1e}, alpha {e1:.1e}, f {rep.f_final:.7g} "
                     f"(oracle {r_orc.f_final:.7g})")
        if flag % 2 == 0:
            assert e0 <= IMG_TOL, notes[-1]
        else:
            # only alpha moves (the clip of flag > 0 applies to both alike)
            np.testing.assert_array_equal(x[0], x_orc[0])
        img = x_orc
    print(f"\nMFS {method} stages: " + "; ".join(notes))


@pytest.mark.parametrize("method", ["CG-FRPRMN", "CG-LBFGS"])
def test_mfs_run_sequence(method):
    """mfs_run(flags 0..3) as one call equals four optimize calls with the
    flags in order; the final objective is printed beside the oracle's."""
    import torch
    data, orc, prob, img = _setup()
    om = "frprmn" if method == "CG-FRPRMN" else "lbfgs"
    d = torch.from_numpy(img.copy()).cuda()
    reps = prob.mfs_run(d, method, iterations=3)
    assert [r.iterations >= 1 for r in reps] == [True] * 4
    x_ref = img.copy()
    for flag in (0, 1, 2, 3):
        x_ref, r_orc = orc.optimize(x_ref, om, iterations=3, flag_opt=flag)
    e = abs(reps[-1].f_final - r_orc.f_final) / abs(r_orc.f_final)
    print(f"\nMFS {method} sequence: f {reps[-1].f_final:.7g}, oracle {r_orc.f_final:.7g}, "
          f"rel {e:.1e}")
    # the same four stages one call at a time
    d2 = torch.from_numpy(img.copy()).cuda()
    for flag in (0, 1, 2, 3):
        prob.optimize(d2, method, iterations=3, flag=flag)
    np.testing.assert_array_equal(d.cpu().numpy(), d2.cpu().numpy())
