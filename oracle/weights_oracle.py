"""FP64 CPU restatement of gpuvmem's weighting schemes (test infrastructure
only): NaturalWeightingScheme::apply (src/naturalweightingscheme.cu:9-52),
UniformWeightingScheme::apply (src/uniformweightingscheme.cu:9-102) and
BriggsWeightingScheme::apply (src/briggsweightingscheme.cu:30-190), for one
field and one correlation, without a uv taper.  Pinned by the reference's
own code through tests/golden/weights_*.npz."""

from __future__ import annotations

import numpy as np

C_LIGHT = np.float32(2.99792458e8)


def cells(uvw_m, freq, M, N, deltau, deltav):
    """Weight-grid cell of every visibility, -1 outside (the first loop of
    each scheme: float wavelength, u < 0 flipped, truncation of
    u / |du| + N/2 + 0.5)."""
    lam = np.float64(np.float32(C_LIGHT / np.float32(freq)))
    u = uvw_m[:, 0] / lam
    v = uvw_m[:, 1] / lam
    neg = u < 0.0
    u = np.where(neg, -u, u)
    v = np.where(neg, -v, v)
    x = np.trunc(u / abs(deltau) + (N // 2) + 0.5).astype(np.int64)
    y = np.trunc(v / abs(deltav) + (M // 2) + 0.5).astype(np.int64)
    ok = (x >= 0) & (y >= 0) & (x < N) & (y < M)
    return np.where(ok, N * y + x, -1)


def _fsum(x, start=np.float32(0.0)):
    """Sequential float32 sum (std::accumulate order), starting at `start`."""
    if len(x) == 0:
        return np.float32(start)
    return np.cumsum(np.concatenate([[np.float32(start)], np.asarray(x, np.float32)]),
                     dtype=np.float32)[-1]


def _fgrid(cell, w, size):
    """Float32 grid of weights summed in visibility order (one thread)."""
    g = np.zeros(size, np.float32)
    ok = cell >= 0
    np.add.at(g, cell[ok], np.asarray(w, np.float32)[ok])
    return g


def apply(scheme, uvw_m, weight, freqs, chan_off, M, N, deltau, deltav, robust=0.0):
    """New weights (float32).  Sums are float32 in the reference's sequential
    order (its result with one OpenMP thread; with more threads the
    reference's own weight grid depends on the thread schedule)."""
    w = np.asarray(weight, np.float32).copy()
    C = len(freqs)
    cl = [cells(uvw_m[chan_off[c]:chan_off[c + 1]], freqs[c], M, N, deltau, deltav)
          for c in range(C)]
    if scheme == "natural":
        return w
    if scheme == "uniform":
        for c in range(C):
            o, e = chan_off[c], chan_off[c + 1]
            ok = cl[c] >= 0
            g = _fgrid(cl[c], weight[o:e], M * N)
            ww = w[o:e]
            ww[:] = np.where(ok, ww / g[np.where(ok, cl[c], 0)], np.float32(0.0))
        return w
    # Briggs: sum of the original weights, channel by channel
    sum_orig = np.float32(0.0)
    for c in range(C):
        sum_orig = np.float32(sum_orig + _fsum(weight[chan_off[c]:chan_off[c + 1]]))
    # first pass: the weights of all channels gridded cumulatively, the
    # squares of the half grid (columns N/2..N-1) summed after each channel
    g = np.zeros(M * N, np.float32)
    sum_sq = np.float32(0.0)
    for c in range(C):
        o, e = chan_off[c], chan_off[c + 1]
        ok = cl[c] >= 0
        np.add.at(g, cl[c][ok], np.asarray(weight[o:e], np.float32)[ok])
        half = g.reshape(M, N)[:, N // 2:].ravel()
        sum_sq = _fsum(half * half, sum_sq)
    average = np.float32(sum_sq / sum_orig)
    r = np.float32(np.float32(5.0) * np.float32(10.0) ** np.float32(-robust))
    f2 = np.float32(np.float32(r * r) / average)
    for c in range(C):
        o, e = chan_off[c], chan_off[c + 1]
        ok = cl[c] >= 0
        gc = _fgrid(cl[c], weight[o:e], M * N)
        den = 1.0 + (gc[np.where(ok, cl[c], 0)] * f2).astype(np.float32).astype(np.float64)
        ww = w[o:e]
        ww[:] = np.where(ok, (ww / den).astype(np.float32), np.float32(0.0))
    return w
