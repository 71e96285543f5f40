"""Writes tests/golden/grid_*.npz: the reference's own convolutional
gridding (do_gridding, with the PillBox2D, Gaussian2D, Sinc2D,
GaussianSinc2D and PSWF_12D kernels and their GCFs; compiled from the
gpuvmem sources by oracle/ref_harness/build_grid.sh, one thread so every
grid cell is summed in a fixed order) applied to seeded synthetic
visibilities.  Run from the repository root in a container that has the
reference sources: python tests/golden/make_grid_golden.py [outdir]"""

import dataclasses
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import refgrid  # noqa: E402
from gpuvmem_gb300 import synth  # noqa: E402

CASES = {
    # the reference's default kernel (src/main.cu: new PillBox2D(), 1 x 1)
    "grid_pillbox_128_2ch": ("pillbox", 1, 1, dict(n=128, nchan=2, seed=41, n_ant=10)),
    "grid_pswf7_64_1ch": ("pswf", 7, 7, dict(n=64, nchan=1, seed=42)),
    "grid_gauss7_64_1ch": ("gaussian", 7, 7, dict(n=64, nchan=1, seed=43)),
    "grid_sinc7_64_2ch": ("sinc", 7, 7, dict(n=64, nchan=2, seed=44)),
    # m != n, and baselines longer than the grid (taps and cells outside)
    "grid_gsinc5x7_32_1ch": ("gaussian_sinc", 5, 7, dict(n=32, nchan=1, seed=45), 2000.0),
    # a channel without visibilities between two with
    "grid_pswf5_64_3ch_empty": ("pswf", 5, 5, dict(n=64, nchan=3, seed=46), None, 1),
}


def main(outdir):
    os.makedirs(outdir, exist_ok=True)
    for name, spec in CASES.items():
        kind, m, n, kw = spec[:4]
        radius = spec[4] if len(spec) > 4 else None
        empty = spec[5] if len(spec) > 5 else None
        cfg = synth.small_config(**kw)
        if radius:
            cfg = dataclasses.replace(cfg, disk_radius_m=radius)
        d = synth.generate(cfg)
        uvw, vo, w, off = d.uvw_m, d.vo, d.weight, np.array(d.chan_off, np.int64)
        if empty is not None:
            o, e = int(off[empty]), int(off[empty + 1])
            keep = np.r_[0:o, e:len(w)]
            uvw, vo, w = uvw[keep], vo[keep], w[keep]
            off = off.copy()
            off[empty + 1:] -= e - o
        r = refgrid.run(kind, uvw, w, vo, d.freqs, off, d.M, d.N, d.DELTAX, d.DELTAY, m=m, n=n)
        counts = np.array([len(c[2]) for c in r["chans"]], np.int64)
        out = dict(kind=kind, m=m, n=n, M=d.M, N=d.N, deltax_deg=d.DELTAX, deltay_deg=d.DELTAY,
                   freqs=np.asarray(d.freqs, np.float32), chan_off=off, uvw_m=uvw,
                   vo=np.asarray(vo, np.float32), weight=np.asarray(w, np.float32),
                   kernel=r["kernel"], support=np.array(r["support"], np.int32),
                   has_gcf=r["gcf"] is not None, counts=counts,
                   out_uvw=np.concatenate([c[0] for c in r["chans"]]),
                   out_vo=np.concatenate([np.stack([c[1].real, c[1].imag], -1)
                                          for c in r["chans"]]).astype(np.float32),
                   out_weight=np.concatenate([c[2] for c in r["chans"]]))
        if r["gcf"] is not None:
            out["gcf"] = r["gcf"]
        np.savez_compressed(os.path.join(outdir, name + ".npz"), **out)
        print(name, kind, (m, n), off.tolist(), counts.tolist())


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(ROOT, "tests", "golden"))
