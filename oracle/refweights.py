"""Runs the reference's own weighting schemes (oracle/_ref/ref_weights, built
by oracle/ref_harness/build_weights.sh from the gpuvmem sources) on numpy
arrays.  Test infrastructure: used to write golden vectors and to time the
reference's CPU path."""

from __future__ import annotations

import os
import struct
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BIN = os.path.join(HERE, "_ref", "ref_weights")
SCHEMES = {"natural": 0, "uniform": 1, "briggs": 2}


def available() -> bool:
    return os.path.exists(BIN)


def run(scheme, uvw_m, weight, freqs, chan_off, M, N, deltau, deltav, robust=0.0, threads=1):
    """Returns (new weights float32 [V], seconds spent in apply())."""
    with tempfile.TemporaryDirectory() as td:
        fin, fout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        with open(fin, "wb") as f:
            f.write(struct.pack("<ifiqqddi", SCHEMES[scheme], float(robust), int(threads), int(M),
                                int(N), float(deltau), float(deltav), len(freqs)))
            for c in range(len(freqs)):
                o, e = int(chan_off[c]), int(chan_off[c + 1])
                f.write(struct.pack("<fq", float(np.float32(freqs[c])), e - o))
                f.write(np.ascontiguousarray(uvw_m[o:e], dtype=np.float64).tobytes())
                f.write(np.ascontiguousarray(weight[o:e], dtype=np.float32).tobytes())
        r = subprocess.run([BIN, fin, fout], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"ref_weights failed ({r.returncode}): {r.stderr}")
        raw = open(fout, "rb").read()
        V = int(chan_off[-1])
        w = np.frombuffer(raw[:4 * V], dtype=np.float32).copy()
        sec = struct.unpack("<d", raw[4 * V:4 * V + 8])[0]
        return w, sec
