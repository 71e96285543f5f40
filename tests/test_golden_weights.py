"""The weighting-scheme oracle against the reference's own Natural, Uniform
and Briggs weighting (golden vectors written by
tests/golden/make_weight_golden.py from the compiled reference sources)."""

import glob
import os

import numpy as np
import pytest

import weights_oracle as WO

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "weights_*.npz")))


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_oracle_matches_reference_weighting(path):
    z = np.load(path)
    w = WO.apply(str(z["scheme"]), z["uvw_m"], z["weight_in"], z["freqs"], z["chan_off"],
                 int(z["M"]), int(z["N"]), float(z["deltau"]), float(z["deltav"]),
                 float(z["robust"]))
    ref = z["weight_out"]
    assert np.array_equal(w == 0, ref == 0)
    assert np.array_equal(w, ref)  # bit for bit with the one-thread reference


def test_golden_files_present():
    assert len(GOLDEN) >= 5
