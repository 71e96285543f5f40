"""Weighting schemes on the GPU against the reference's own weighting (one
thread), bit for bit."""

import ctypes as C
import glob
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "weights_*.npz")))
SCHEME = {"natural": 0, "uniform": 1, "briggs": 2}


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_gpu_weighting_matches_reference(path):
    import gpuvmem_gb300 as gv
    z = np.load(path)
    out = gv.apply_weighting(str(z["scheme"]), float(z["robust"]), int(z["M"]), int(z["N"]),
                             float(z["deltax_deg"]), float(z["deltay_deg"]), z["freqs"],
                             z["chan_off"], z["uvw_m"], z["weight_in"])
    assert np.array_equal(out, z["weight_out"])
