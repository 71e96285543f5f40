"""CPU restatement of gpuvmem's convolutional gridding (test infrastructure
only): the convolution-kernel and gridding-correction tables of the CKernel
family (src/pillBox2D.cu, src/gaussian2D.cu, src/sinc2D.cu,
src/gaussianSinc2D.cu, src/pswf_12D.cu; set up as src/mfs.cu:510-516) in
FP64 rounded to FP32, and do_gridding (src/functions.cu:1339-1653) with the
one-thread order of its FP32 sums.  Pinned by the reference's own code
through tests/golden/grid_*.npz."""

from __future__ import annotations

import math

import numpy as np

C_LIGHT = np.float32(2.99792458e8)
RPDEG = math.pi / 180.0
PI_F = float(np.float32(math.pi))

# Schwab (1984) rational approximation of the spheroidal function (support 6,
# alpha 1), the coefficients src/pswf_12D.cu uses
_P = ((8.203343e-2, -3.644705e-1, 6.278660e-1, -5.335581e-1, 2.312756e-1),
      (4.028559e-3, -3.697768e-2, 1.021332e-1, -1.201436e-1, 6.412774e-2))
_Q = ((1.0, 8.212018e-1, 2.078043e-1), (1.0, 9.599102e-1, 2.918724e-1))

DEFAULTS = {  # (w, alpha, w2) of the (m, n) constructors
    "pillbox": (1.0, 2.0, 1.55), "gaussian": (1.0, 2.0, 1.55), "sinc": (1.0, 2.0, 1.55),
    "gaussian_sinc": (2.52, 2.0, 1.55), "pswf": (6.0, 2.0, 1.55)}


def _gauss(x, y, sx, sy, w, alpha):
    rx, ry = abs(x), abs(y)
    if rx < w * sx and ry < w * sy:
        return math.exp(-((rx / (w * sx)) ** alpha + (ry / (w * sy)) ** alpha))
    return 0.0


def _sinc1(x, sigma, w):
    r = abs(x)
    if r >= w * sigma:
        return 0.0
    v = r / (w * sigma)
    return 1.0 if v == 0.0 else math.sin(math.pi * v) / (math.pi * v)


def _pswf_rational(nu):
    a = abs(nu)
    if a > 1.0:
        return 0.0
    part = 0 if a < 0.75 else 1
    d = a * a - (0.75 if part == 0 else 1.0) ** 2
    top = sum(_P[part][i] * d ** i for i in range(5))
    bottom = sum(_Q[part][i] * d ** i for i in range(3))
    return top / bottom if bottom > 0.0 else 0.0


def _pswf1(x, sigma, w):
    nu = abs(x) / (w * sigma)
    if nu == 0.0:
        return 1.0
    return (1.0 - nu * nu) * _pswf_rational(nu)


def kernel_table(kind, m, n, deltau, deltav, w=None, alpha=None, w2=None):
    """(table [m, n] float32, support) as buildKernel with sigmas |deltau|,
    |deltav| (both supports are floor(m/2))."""
    dw, da, dw2 = DEFAULTS[kind]
    w = dw if w is None else w
    alpha = da if alpha is None else alpha
    w2 = dw2 if w2 is None else w2
    sx, sy = float(np.float32(abs(deltau))), float(np.float32(abs(deltav)))
    sup = m // 2
    t = np.zeros((m, n), np.float64)
    for i in range(m):
        for j in range(n):
            y, x = (i - sup) * sy, (j - sup) * sx
            if kind == "pillbox":
                t[i, j] = float(abs(x) < (m / 2.0) * sx) * float(abs(y) < (n / 2.0) * sy)
            elif kind == "gaussian":
                t[i, j] = _gauss(x, y, sx, sy, w, alpha)
            elif kind == "sinc":
                # Sinc2D::buildKernel fills sinc2D's (x, x0, y, y0) slots with
                # (x, y, 0, 0): sinc(|x - y|) * sinc(0)
                t[i, j] = _sinc1(x - y, sx, w)
            elif kind == "gaussian_sinc":
                t[i, j] = _gauss(x, y, sx, sy, w, alpha) * _sinc1(x, sx, w2) * _sinc1(y, sy, w2)
            else:
                t[i, j] = _pswf1(x, sx, w) * _pswf1(y, sy, w)
    return t.astype(np.float32), (sup, sup)


def gcf_table(kind, M, N, deltax_deg, deltay_deg, alpha=2.0):
    """The M x N gridding correction function (initializeGCF: w = M, cell
    sizes |deltax|, |deltay| in radians), or None for Sinc2D and
    GaussianSinc2D, which define none."""
    if kind in ("sinc", "gaussian_sinc"):
        return None
    if kind == "pillbox":
        return np.ones((M, N), np.float32)
    sx = float(np.float32(abs(RPDEG * deltax_deg)))
    sy = float(np.float32(abs(RPDEG * deltay_deg)))
    sup, w = M // 2, float(M)
    g = np.zeros((M, N), np.float64)
    for i in range(M):
        y = (i - sup) * sy
        for j in range(N):
            x = (j - sup) * sx
            if kind == "gaussian":
                g[i, j] = _gauss(PI_F * x, PI_F * y, sx, sy, 2.0 * w, alpha)
            else:
                g[i, j] = 1.0 / (_pswf1(x, sx, w) * _pswf1(y, sy, w))
    return g.astype(np.float32)


def grid_channel(table, support, uvw_m, vo, weight, freq, M, N, deltax_deg, deltay_deg):
    """do_gridding for one channel: (uvw [k, 3] f64 metres, vo [k] c64,
    weight [k] f32) of the occupied cells in row-major order."""
    km, kn = table.shape
    sx, sy = support
    deltau = 1.0 / (M * (RPDEG * deltax_deg))
    deltav = 1.0 / (N * (RPDEG * deltay_deg))
    cj, ck = math.floor(N / 2.0), math.floor(M / 2.0)
    lam = np.float32(C_LIGHT / np.float32(freq))
    n = len(weight)
    uvw = np.asarray(uvw_m, np.float64)
    u = np.concatenate([uvw[:, 0], uvw[:, 0] * -1.0])
    v = np.concatenate([uvw[:, 1], uvw[:, 1] * -1.0])
    vo = np.asarray(vo)
    if not np.iscomplexobj(vo):  # [k, 2] float pairs
        vo = vo[:, 0].astype(np.float32) + 1j * vo[:, 1].astype(np.float32)
    vo = vo.astype(np.complex64)
    vr = np.concatenate([vo.real, vo.real]).astype(np.float32)
    vi = np.concatenate([vo.imag, vo.imag * np.float32(-1.0)]).astype(np.float32)
    w = np.concatenate([weight, weight]).astype(np.float32)
    j = np.trunc((u / np.float64(lam) / deltau + cj) + 0.5).astype(np.int64)
    k = np.trunc((v / np.float64(lam) / deltav + ck) + 0.5).astype(np.int64)
    # every (visibility, tap) in the reference's loop order: visibility-major
    cells, kv, zi = [], [], []
    for mm in range(-sy, sy + 1):
        for nn in range(-sx, sx + 1):
            sk, sj, ki, kj = k + mm, j + nn, mm + sy, nn + sx
            ok = (sk >= 0) & (sk < M) & (sj >= 0) & (sj < N) & (ki < km) & (kj < kn)
            cells.append(np.where(ok, N * sk + sj, -1))
            kv.append(np.full(2 * n, table[ki, kj] if (ki < km and kj < kn) else 0.0,
                              np.float32))
            zi.append(np.arange(2 * n))
    cells = np.stack(cells, 1).reshape(-1)
    kv = np.stack(kv, 1).reshape(-1)
    zi = np.stack(zi, 1).reshape(-1)
    keep = cells >= 0
    cells, kv, zi = cells[keep], kv[keep], zi[keep]
    MN = M * N
    gw = np.zeros(MN, np.float32)
    ga = np.zeros(MN, np.float32)
    gr = np.zeros(MN, np.float32)
    gi = np.zeros(MN, np.float32)
    wz = w[zi]
    np.add.at(gw, cells, wz * kv)
    np.add.at(ga, cells, wz * (kv * kv))
    np.add.at(gr, cells, (wz * vr[zi]) * kv)
    np.add.at(gi, cells, (wz * vi[zi]) * kv)
    occ = (ga != 0) & (gw != 0)
    with np.errstate(divide="ignore", invalid="ignore"):
        weff = np.where(occ, (gw * gw) / ga, np.float32(0.0)).astype(np.float32)
        orr = np.where(occ, gr / gw, np.float32(0.0)).astype(np.float32)
        oii = np.where(occ, gi / gw, np.float32(0.0)).astype(np.float32)
    sel = np.nonzero(weff > 0)[0]
    gj, gk = sel % N, sel // N
    ouvw = np.zeros((len(sel), 3), np.float64)
    ouvw[:, 0] = ((gj - cj) * deltau) * np.float64(lam)
    ouvw[:, 1] = ((gk - ck) * deltav) * np.float64(lam)
    return ouvw, (orr[sel] + 1j * oii[sel]).astype(np.complex64), weff[sel]
