"""Writes tests/golden/weights_*.npz: the reference's own Natural, Uniform
and Briggs weighting schemes (compiled from the gpuvmem sources by
oracle/ref_harness/build_weights.sh, one thread so the weight gridding is
summed in a fixed order) applied to seeded synthetic visibilities.
Run from the repository root in a container that has the reference
sources: python tests/golden/make_weight_golden.py [outdir]"""

import math
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import refweights  # noqa: E402
from gpuvmem_gb300 import synth  # noqa: E402

CASES = {
    "weights_uniform_64_3ch": ("uniform", 0.0, dict(n=64, nchan=3, seed=31)),
    "weights_briggs0_64_3ch": ("briggs", 0.0, dict(n=64, nchan=3, seed=32)),
    "weights_briggs1_128_2ch": ("briggs", 1.0, dict(n=128, nchan=2, seed=33, n_ant=12)),
    "weights_briggsm1_64_1ch": ("briggs", -1.0, dict(n=64, nchan=1, seed=34)),
    "weights_natural_64_2ch": ("natural", 0.0, dict(n=64, nchan=2, seed=35)),
}


def main(outdir):
    os.makedirs(outdir, exist_ok=True)
    for name, (scheme, robust, kw) in CASES.items():
        cfg = synth.small_config(**kw)
        d = synth.generate(cfg)
        # src/mfs.cu:531-534: deltax = RPDEG_D * DELTAX, deltau = 1 / (M * deltax)
        dx = (math.pi / 180.0) * d.DELTAX
        dy = (math.pi / 180.0) * d.DELTAY
        deltau, deltav = 1.0 / (d.M * dx), 1.0 / (d.N * dy)
        w, _ = refweights.run(scheme, d.uvw_m, d.weight, d.freqs, d.chan_off, d.M, d.N, deltau,
                              deltav, robust, threads=1)
        np.savez_compressed(os.path.join(outdir, name + ".npz"), scheme=scheme, robust=robust,
                            M=d.M, N=d.N, deltau=deltau, deltav=deltav, deltax_deg=d.DELTAX,
                            deltay_deg=d.DELTAY, freqs=d.freqs,
                            chan_off=d.chan_off, uvw_m=d.uvw_m, weight_in=d.weight,
                            weight_out=w)
        print(name, scheme, robust, int(d.chan_off[-1]), float(w.min()), float(w.max()))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(ROOT, "tests", "golden"))
