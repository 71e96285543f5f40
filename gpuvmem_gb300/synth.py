"""Seeded synthetic interferometric data sets.

The reference reads visibilities from casacore Measurement Sets; here the same
structures (one field, one XX correlation per channel, u,v,w in metres,
complex visibilities, weights) are generated from a seeded array layout, an
hour-angle track and a sky of elliptical Gaussian components with analytic
Fourier transforms.  Conventions follow the reference's forward model:
x = (j - x0) * DELTAX (radians), Vo = sum_s S_s A(x_s) G_s(u, v)
exp(+2 pi i (u x_s + v y_s)), DELTAX negative, crpix = N/2 + 1 so that the
phase centre is pixel N/2.

Natural weights are 1/sigma^2; Briggs weighting restates
BriggsWeightingScheme::apply (src/briggsweightingscheme.cu:30-190),
including its cumulative gridding of weights across channels in the first
pass.
"""

from __future__ import annotations

import dataclasses
import math
from typing import List, Optional

import numpy as np

C_LIGHT = np.float32(2.99792458e8)
RPDEG = math.pi / 180.0
RPARCSEC = math.pi / (180.0 * 3600.0)
SITE_LAT_DEG = -23.0


@dataclasses.dataclass
class SynthConfig:
    name: str
    n: int                       # image is n x n
    cell_arcsec: float
    n_ant: int
    disk_radius_m: float
    freqs_hz: List[float]
    dec_deg: float
    ha_start_h: float
    ha_stop_h: float
    dt_s: float
    sigma_jy: float = 1e-3
    n_sources: int = 20
    flux_range_jy: tuple = (1e-3, 50e-3)
    fwhm_range_arcsec: tuple = (0.1, 1.0)
    point_source_jy: float = 0.0
    pb_fwhm_arcsec: float = 25.0
    antenna_diameter: float = 12.0
    weighting: str = "natural"   # or "briggs"
    robust: float = 0.0
    source_radius_frac: float = 0.3
    flag_fraction_range: tuple = (0.0, 0.0)
    alpha_range: Optional[tuple] = None
    seed: int = 0
    array_seed: Optional[int] = None  # antenna layout seed (default: seed)


CONFIG0 = SynthConfig(
    name="plain-mem-256", n=256, cell_arcsec=0.05, n_ant=30, disk_radius_m=500.0,
    freqs_hz=[230e9], dec_deg=-30.0, ha_start_h=-2.0, ha_stop_h=2.0, dt_s=60.0,
    n_sources=20, seed=1)

CONFIG1 = SynthConfig(
    name="plain-mem-2048-8ch", n=2048, cell_arcsec=0.01, n_ant=50,
    disk_radius_m=2000.0, freqs_hz=list(np.linspace(225e9, 235e9, 8)),
    dec_deg=-30.0, ha_start_h=-2.0, ha_stop_h=2.0, dt_s=4.0, n_sources=200,
    point_source_jy=1.0, weighting="briggs", robust=0.0, seed=2)

# 4 spectral windows x 16 channels, 85-115 GHz, per-channel flag fraction
# U(0, 0.4), spectral indices U(-1, 3): the batched MFS workload
CONFIG2 = SynthConfig(
    name="mfs-1024-64ch", n=1024, cell_arcsec=0.05, n_ant=40, disk_radius_m=1000.0,
    freqs_hz=[f for spw in range(4) for f in np.linspace(85e9 + spw * 7.5e9,
                                                          85e9 + spw * 7.5e9 + 7.0e9, 16)],
    dec_deg=-30.0, ha_start_h=-1.0, ha_stop_h=1.0, dt_s=10.0, n_sources=40,
    pb_fwhm_arcsec=40.0, flag_fraction_range=(0.0, 0.4), alpha_range=(-1.0, 3.0), seed=22)


def small_config(n=64, n_ant=8, n_times=40, nchan=1, seed=0, pb_fwhm_frac=0.45,
                 weighting="natural", n_sources=6) -> SynthConfig:
    """A problem the FP64 oracle evaluates in well under a second.  The
    primary beam is narrow relative to the field so the noise mask and the
    beam cut-off both fall inside the image."""
    cell = 0.05
    fwhm = pb_fwhm_frac * n * cell
    span = 4.0
    return SynthConfig(
        name=f"small-{n}", n=n, cell_arcsec=cell, n_ant=n_ant,
        disk_radius_m=150.0 * n / 64.0, freqs_hz=list(np.linspace(229e9, 231e9, nchan)),
        dec_deg=-30.0, ha_start_h=-span / 2, ha_stop_h=span / 2,
        dt_s=span * 3600.0 / n_times, n_sources=n_sources, pb_fwhm_arcsec=fwhm,
        weighting=weighting, seed=seed, source_radius_frac=0.2)


@dataclasses.dataclass
class SynthData:
    cfg: SynthConfig
    M: int
    N: int
    DELTAX: float
    DELTAY: float
    crpix1: float
    crpix2: float
    xobs: float
    yobs: float
    nu_0: float
    antenna_diameter: float
    pb_factor: float
    pb_cutoff: float
    primary_beam: int              # 0 airy, 1 gaussian (reference enum order)
    freqs: np.ndarray              # float32 [C]
    chan_off: np.ndarray           # int64 [C+1]
    uvw_m: np.ndarray              # float64 [V,3] metres, as observed
    vo: np.ndarray                 # float32 [V,2]
    weight: np.ndarray             # float32 [V]
    sources: dict

    @property
    def nvis(self) -> int:
        return int(self.chan_off[-1])


def _array_enu(rng, n_ant, radius):
    r = radius * np.sqrt(rng.uniform(0.0, 1.0, n_ant))
    th = rng.uniform(0.0, 2.0 * math.pi, n_ant)
    return np.stack([r * np.cos(th), r * np.sin(th), np.zeros(n_ant)], axis=1)


def baseline_uvw(cfg: SynthConfig, rng) -> np.ndarray:
    """u,v,w (metres) for all baselines and integrations, time-major."""
    enu = _array_enu(rng, cfg.n_ant, cfg.disk_radius_m)
    i, j = np.triu_indices(cfg.n_ant, k=1)
    d = enu[j] - enu[i]
    lat = SITE_LAT_DEG * RPDEG
    X = -math.sin(lat) * d[:, 1] + math.cos(lat) * d[:, 2]
    Y = d[:, 0]
    Z = math.cos(lat) * d[:, 1] + math.sin(lat) * d[:, 2]
    n_t = int(round((cfg.ha_stop_h - cfg.ha_start_h) * 3600.0 / cfg.dt_s))
    H = (cfg.ha_start_h * 3600.0 + np.arange(n_t) * cfg.dt_s) / 3600.0 * 15.0 * RPDEG
    dec = cfg.dec_deg * RPDEG
    sH, cH = np.sin(H)[:, None], np.cos(H)[:, None]
    u = sH * X + cH * Y
    v = -math.sin(dec) * cH * X + math.sin(dec) * sH * Y + math.cos(dec) * Z
    w = math.cos(dec) * cH * X - math.cos(dec) * sH * Y + math.sin(dec) * Z
    return np.stack([u.ravel(), v.ravel(), w.ravel()], axis=1)


def _sources(cfg: SynthConfig, rng, DELTAX_rad, DELTAY_rad, x0, y0):
    ns = cfg.n_sources
    lo, hi = cfg.flux_range_jy
    flux = np.exp(rng.uniform(math.log(lo), math.log(hi), ns))
    fmaj = rng.uniform(*cfg.fwhm_range_arcsec, ns) * RPARCSEC
    fmin = fmaj * rng.uniform(0.3, 1.0, ns)
    pa = rng.uniform(0.0, math.pi, ns)
    rad = cfg.source_radius_frac * cfg.n * np.sqrt(rng.uniform(0, 1, ns))
    th = rng.uniform(0, 2 * math.pi, ns)
    px = np.round(x0 + rad * np.cos(th))
    py = np.round(y0 + rad * np.sin(th))
    if cfg.point_source_jy > 0:
        flux = np.append(flux, cfg.point_source_jy)
        fmaj = np.append(fmaj, 0.0)
        fmin = np.append(fmin, 0.0)
        pa = np.append(pa, 0.0)
        px = np.append(px, x0 + 3)
        py = np.append(py, y0 - 5)
    alpha = None
    if cfg.alpha_range is not None:
        alpha = rng.uniform(*cfg.alpha_range, flux.size)
    return dict(flux=flux, fmaj=fmaj, fmin=fmin, pa=pa,
                x=(px - int(x0)) * DELTAX_rad, y=(py - int(y0)) * DELTAY_rad,
                px=px, py=py, alpha=alpha)


def gaussian_beam(r_rad, fwhm_rad):
    return np.exp(-4.0 * math.log(2.0) * (r_rad / fwhm_rad) ** 2)


def _sky_vis_numpy(u, v, src, atten, nu, nu0, chunk=1 << 20):
    out = np.zeros((u.size, 2), dtype=np.float64)
    k = math.pi ** 2 / (4.0 * math.log(2.0))
    for s in range(src["flux"].size):
        S = src["flux"][s] * atten[s]
        if src["alpha"] is not None:
            S *= (nu / nu0) ** src["alpha"][s]
        cp, sp = math.cos(src["pa"][s]), math.sin(src["pa"][s])
        for a in range(0, u.size, chunk):
            uu, vv = u[a:a + chunk], v[a:a + chunk]
            up = uu * cp - vv * sp
            vp = uu * sp + vv * cp
            amp = S * np.exp(-k * ((src["fmaj"][s] * up) ** 2 + (src["fmin"][s] * vp) ** 2))
            ph = 2.0 * math.pi * (uu * src["x"][s] + vv * src["y"][s])
            out[a:a + chunk, 0] += amp * np.cos(ph)
            out[a:a + chunk, 1] += amp * np.sin(ph)
    return out


def _sky_vis_torch(u, v, src, atten, nu, nu0, device):
    import torch
    uu = torch.from_numpy(u).to(device)
    vv = torch.from_numpy(v).to(device)
    re = torch.zeros_like(uu)
    im = torch.zeros_like(uu)
    k = math.pi ** 2 / (4.0 * math.log(2.0))
    for s in range(src["flux"].size):
        S = float(src["flux"][s] * atten[s])
        if src["alpha"] is not None:
            S *= float((nu / nu0) ** src["alpha"][s])
        cp, sp = math.cos(src["pa"][s]), math.sin(src["pa"][s])
        up = uu * cp - vv * sp
        vp = uu * sp + vv * cp
        amp = S * torch.exp(-k * ((float(src["fmaj"][s]) * up) ** 2 + (float(src["fmin"][s]) * vp) ** 2))
        ph = 2.0 * math.pi * (uu * float(src["x"][s]) + vv * float(src["y"][s]))
        re += amp * torch.cos(ph)
        im += amp * torch.sin(ph)
    return torch.stack([re, im], dim=1).cpu().numpy()


def briggs_weights(uvw_m, weight, freqs, chan_off, M, N, deltau, deltav, robust):
    """BriggsWeightingScheme::apply, src/briggsweightingscheme.cu:30-190."""
    w = weight.astype(np.float32).copy()
    sum_orig = np.float32(np.sum(weight, dtype=np.float64))
    g = np.zeros(M * N, dtype=np.float64)
    sum_sq = 0.0
    cells = []
    for c in range(len(freqs)):
        o, e = chan_off[c], chan_off[c + 1]
        lam = np.float32(C_LIGHT / np.float32(freqs[c]))
        ux = uvw_m[o:e, 0] / np.float64(lam)
        uy = uvw_m[o:e, 1] / np.float64(lam)
        neg = ux < 0.0
        ux = np.where(neg, -ux, ux)
        uy = np.where(neg, -uy, uy)
        gx = ux / abs(deltau)
        gy = uy / abs(deltav)
        x = np.trunc(gx + (N // 2) + 0.5).astype(np.int64)
        y = np.trunc(gy + (M // 2) + 0.5).astype(np.int64)
        ok = (x >= 0) & (y >= 0) & (x < N) & (y < M)
        cell = np.where(ok, N * y + x, -1)
        cells.append(cell)
        g += np.bincount(cell[ok], weights=weight[o:e][ok].astype(np.float64), minlength=M * N)
        gg = g.reshape(M, N)[:, N // 2:]
        sum_sq += float(np.sum(gg * gg))
    avg = np.float32(sum_sq) / sum_orig
    f2 = np.float32((5.0 * 10.0 ** (-robust)) ** 2) / avg
    for c in range(len(freqs)):
        o, e = chan_off[c], chan_off[c + 1]
        cell = cells[c]
        ok = cell >= 0
        gc = np.bincount(cell[ok], weights=weight[o:e][ok].astype(np.float64), minlength=M * N)
        ww = w[o:e]
        den = 1.0 + gc[np.where(ok, cell, 0)] * np.float64(f2)
        ww[:] = np.where(ok, ww / den, 0.0).astype(np.float32)
    return w


def generate(cfg: SynthConfig, device: Optional[str] = None) -> SynthData:
    """Build the synthetic data set.  ``device`` = a torch CUDA device
    evaluates the sky visibilities there (large configurations); the default
    evaluates them with numpy."""
    rng_array = np.random.default_rng([cfg.seed if cfg.array_seed is None else cfg.array_seed, 1])
    rng_sky = np.random.default_rng([cfg.seed, 2])
    rng_noise = np.random.default_rng([cfg.seed, 3])
    rng_flag = np.random.default_rng([cfg.seed, 4])
    n = cfg.n
    DELTAX = -cfg.cell_arcsec / 3600.0
    DELTAY = cfg.cell_arcsec / 3600.0
    crpix = n / 2 + 1.0
    x0 = y0 = crpix - 1.0
    nu_0 = np.float32(0.5 * (max(cfg.freqs_hz) + min(cfg.freqs_hz)))
    lam0 = float(C_LIGHT / nu_0)
    pb_factor = np.float32(cfg.pb_fwhm_arcsec * RPARCSEC * cfg.antenna_diameter / lam0)
    lam_max = float(C_LIGHT / np.float32(min(cfg.freqs_hz)))
    pb_cutoff = np.float32(pb_factor * (lam_max / cfg.antenna_diameter))
    base = baseline_uvw(cfg, rng_array)
    src = _sources(cfg, rng_sky, DELTAX * RPDEG, DELTAY * RPDEG, x0, y0)
    uvws, vos, ws, offs = [], [], [0], None
    counts = []
    for c, f in enumerate(cfg.freqs_hz):
        f32 = np.float32(f)
        lam = float(C_LIGHT / f32)
        fwhm = float(pb_factor) * lam / cfg.antenna_diameter
        r = np.hypot(src["x"], src["y"])
        atten = gaussian_beam(r, fwhm)
        uvw = base.copy()
        lo, hi = cfg.flag_fraction_range
        if hi > 0:
            frac = rng_flag.uniform(lo, hi)
            keep = rng_flag.uniform(0, 1, uvw.shape[0]) >= frac
            uvw = uvw[keep]
        u_l, v_l = uvw[:, 0] / lam, uvw[:, 1] / lam
        if device is not None and device != "cpu":
            vis = _sky_vis_torch(u_l, v_l, src, atten, float(f32), float(nu_0), device)
        else:
            vis = _sky_vis_numpy(u_l, v_l, src, atten, float(f32), float(nu_0))
        vis += rng_noise.normal(0.0, cfg.sigma_jy, vis.shape)
        uvws.append(uvw)
        vos.append(vis.astype(np.float32))
        counts.append(uvw.shape[0])
    chan_off = np.zeros(len(counts) + 1, dtype=np.int64)
    chan_off[1:] = np.cumsum(counts)
    uvw_m = np.concatenate(uvws, axis=0)
    vo = np.concatenate(vos, axis=0)
    weight = np.full(uvw_m.shape[0], np.float32(1.0 / cfg.sigma_jy ** 2), dtype=np.float32)
    freqs = np.array([np.float32(f) for f in cfg.freqs_hz], dtype=np.float32)
    if cfg.weighting == "briggs":
        deltau = 1.0 / (n * (DELTAX * RPDEG))
        deltav = 1.0 / (n * (DELTAY * RPDEG))
        weight = briggs_weights(uvw_m, weight, freqs, chan_off, n, n, deltau, deltav, cfg.robust)
    return SynthData(
        cfg=cfg, M=n, N=n, DELTAX=DELTAX, DELTAY=DELTAY, crpix1=crpix, crpix2=crpix,
        xobs=float(np.float32(x0)), yobs=float(np.float32(y0)), nu_0=float(nu_0),
        antenna_diameter=cfg.antenna_diameter, pb_factor=float(pb_factor),
        pb_cutoff=float(pb_cutoff), primary_beam=1, freqs=freqs, chan_off=chan_off,
        uvw_m=np.ascontiguousarray(uvw_m), vo=np.ascontiguousarray(vo),
        weight=weight, sources=src)


def config3_problems(count: int = 64, seed: int = 3):
    """Configuration 3: `count` independent problems with image sides drawn
    from {128, 256, 512}, visibility counts log-uniform in [20k, 500k], 10-40
    antennas, one channel at U(100, 300) GHz, their own skies, and an entropy
    factor log-uniform in [1e-3, 1e-1].  Returns (configs, entropy factors)."""
    rng = np.random.default_rng([seed, 99])
    cfgs, lams = [], []
    for k in range(count):
        n = int(rng.choice([128, 256, 512]))
        nvis = float(np.exp(rng.uniform(math.log(20e3), math.log(500e3))))
        n_ant = int(rng.integers(10, 41))
        nbl = n_ant * (n_ant - 1) // 2
        n_t = max(4, int(round(nvis / nbl)))
        freq = float(rng.uniform(100e9, 300e9))
        cell = 0.05 * 230e9 / freq
        span = 4.0
        cfgs.append(SynthConfig(
            name=f"batch-{k}-{n}", n=n, cell_arcsec=cell, n_ant=n_ant,
            disk_radius_m=500.0, freqs_hz=[freq], dec_deg=-30.0, ha_start_h=-span / 2,
            ha_stop_h=span / 2, dt_s=span * 3600.0 / n_t, n_sources=int(rng.integers(5, 30)),
            pb_fwhm_arcsec=0.45 * n * cell, seed=1000 + k, source_radius_frac=0.2))
        lams.append(float(np.exp(rng.uniform(math.log(1e-3), math.log(1e-1)))))
    return cfgs, lams
