"""Runs the reference's own convolutional gridding and convolution-kernel /
GCF tables (oracle/_ref/ref_grid, built by oracle/ref_harness/build_grid.sh
from the gpuvmem sources) on numpy arrays.  Test infrastructure: used to
write golden vectors and to time the reference's CPU path."""

from __future__ import annotations

import os
import struct
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BIN = os.path.join(HERE, "_ref", "ref_grid")
KINDS = {"pillbox": 0, "gaussian": 1, "sinc": 2, "gaussian_sinc": 3, "pswf": 4}


def available() -> bool:
    return os.path.exists(BIN)


def run(kind, uvw_m, weight, vo, freqs, chan_off, M, N, deltax_deg, deltay_deg, m=7, n=7,
        threads=1):
    """Returns dict(kernel [km, kn], support (sx, sy), gcf [M, N] or None,
    chans: list of (uvw [k, 3] f64, vo [k] c64, weight [k] f32), seconds)."""
    vo = np.asarray(vo)
    vo2 = np.stack([vo.real, vo.imag], -1).astype(np.float32) if np.iscomplexobj(vo) else \
        np.ascontiguousarray(vo, dtype=np.float32)
    with tempfile.TemporaryDirectory() as td:
        fin, fout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        with open(fin, "wb") as f:
            f.write(struct.pack("<iiiiqqddi", KINDS[kind], int(m), int(n), int(threads), int(M),
                                int(N), float(deltax_deg), float(deltay_deg), len(freqs)))
            for c in range(len(freqs)):
                o, e = int(chan_off[c]), int(chan_off[c + 1])
                f.write(struct.pack("<fq", float(np.float32(freqs[c])), e - o))
                f.write(np.ascontiguousarray(uvw_m[o:e], dtype=np.float64).tobytes())
                f.write(np.ascontiguousarray(weight[o:e], dtype=np.float32).tobytes())
                f.write(np.ascontiguousarray(vo2[o:e], dtype=np.float32).tobytes())
        r = subprocess.run([BIN, fin, fout], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"ref_grid failed ({r.returncode}): {r.stderr}")
        raw = open(fout, "rb").read()
    pos = 0

    def take(dtype, count):
        nonlocal pos
        a = np.frombuffer(raw, dtype=dtype, count=count, offset=pos).copy()
        pos += a.nbytes
        return a

    km, kn, sx, sy = (int(x) for x in take(np.int32, 4))
    kernel = take(np.float32, km * kn).reshape(km, kn)
    has_gcf = int(take(np.int32, 1)[0])
    gcf = take(np.float32, M * N).reshape(M, N) if has_gcf else None
    chans = []
    for _ in range(len(freqs)):
        cnt = int(take(np.int64, 1)[0])
        uvw = take(np.float64, 3 * cnt).reshape(cnt, 3)
        v = take(np.float32, 2 * cnt).reshape(cnt, 2)
        w = take(np.float32, cnt)
        chans.append((uvw, v[:, 0] + 1j * v[:, 1].astype(np.complex64), w))
    sec = float(take(np.float64, 1)[0])
    return dict(kernel=kernel, support=(sx, sy), gcf=gcf, chans=chans, seconds=sec)
