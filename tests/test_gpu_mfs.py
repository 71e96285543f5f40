"""The two-image MFS fit (I_nu0 and spectral index alpha) solved with
MFS::run's flag sequence 0, 1, 2, 3 (src/mfs.cu:999-1008), against the FP64
oracle's optimiser: each stage starts both from the image the oracle's
previous stage left, runs the stage's iterations, and the two images agree
within 1e-4 of each plane's peak."""

import numpy as np
import pytest

import oracle as O
from gpuvmem_gb300 import synth

pytestmark = pytest.mark.gpu

IMG_TOL = 1e-4
TERMS = [(O.FI_CHI2, 1.0, 0, 0, 0.0, 0.0, 0.0), (O.FI_ENTROPY, 0.01, 0, 0, 0.001, -1.0, 0.0)]


@pytest.mark.parametrize("method", ["CG-FRPRMN", "CG-LBFGS"])
def test_mfs_four_flag_sequence(method):
    import dataclasses
    import torch
    import gpuvmem_gb300 as gv
    cfg = dataclasses.replace(synth.small_config(n=64, n_ant=10, n_times=40, nchan=4, seed=31),
                              freqs_hz=list(np.linspace(85e9, 115e9, 4)), alpha_range=(-1.0, 3.0))
    data = synth.generate(cfg)
    orc = O.Oracle(data, TERMS)
    prob = gv.Problem(data, [tuple(t) for t in TERMS])
    img = orc.initial_image()
    errs = []
    for flag in (0, 1, 2, 3):
        iters = 2 if flag % 2 == 0 else 1
        x_orc, _ = orc.optimize(img.copy(), "frprmn" if method == "CG-FRPRMN" else "lbfgs",
                                iterations=iters, flag_opt=flag)
        d = torch.from_numpy(img.copy()).cuda()
        reps = prob.mfs_run(d, method, iterations=iters, flags=(flag,))
        assert reps[0].iterations >= 1
        x = d.cpu().numpy()
        e = [np.abs(x[p] - x_orc[p]).max() / max(np.abs(x_orc[p]).max(), 1e-30) for p in (0, 1)]
        errs.append(e)
        assert e[0] <= IMG_TOL and e[1] <= IMG_TOL, (flag, e)
        img = x_orc
    print(f"\nMFS {method} flags 0-3: image errors (I_nu0, alpha) of the peak: "
          + "; ".join(f"{a:.1e}, {b:.1e}" for a, b in errs))
    # the alpha plane moved: the sequence fitted the spectral index
    assert np.abs(img[1]).max() > 0
