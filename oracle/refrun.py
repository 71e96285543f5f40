"""ctypes binding of the reference harness (ref_harness/refrun.cpp).

TEST INFRASTRUCTURE ONLY: runs the reference's own CUDA kernels (compiled
from the reference sources into oracle/_ref/ref_kernels.cubin) with the
reference's launch sequence, to pin the CPU oracle and to time the
reference CUDA build.  Needs a GPU and the prebuilt cubin.
"""

from __future__ import annotations

import ctypes as C
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
CUBIN = os.path.join(_HERE, "_ref", "ref_kernels.cubin")
_LIB = None


def available() -> bool:
    return os.path.exists(CUBIN) and os.path.exists(os.path.join(_HERE, "librefrun.so"))


def lib():
    global _LIB
    if _LIB is None:
        L = C.CDLL(os.path.join(_HERE, "librefrun.so"))
        f32p, f64p, i64p = C.POINTER(C.c_float), C.POINTER(C.c_double), C.POINTER(C.c_long)
        vp = C.c_void_p
        L.rr_last_error.restype = C.c_char_p
        L.rr_load.argtypes = [C.c_char_p]
        L.rr_create.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_float, C.c_float,
                                C.c_float, C.c_float, C.c_float, C.c_float, C.c_int, C.c_float,
                                C.c_float, C.c_float, C.c_float, C.c_float, C.c_int, C.c_int,
                                f32p, i64p, f64p, f32p, f32p, C.POINTER(vp)]
        L.rr_info.argtypes = [vp, f32p, f32p, f32p]
        L.rr_chi2.argtypes = [vp, f32p, C.c_int, f32p]
        L.rr_dchi2.argtypes = [vp, f32p, C.c_int, f32p]
        L.rr_residuals.argtypes = [vp, f32p]
        L.rr_prior.argtypes = [vp, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float, C.c_int,
                               f32p, f32p, f32p]
        L.rr_time.argtypes = [vp, f32p, C.c_int, C.c_int, f64p, f64p]
        L.rr_dchi2_band.argtypes = [vp, f32p, C.c_int, C.c_int, C.c_int, f32p]
        L.rr_destroy.argtypes = [vp]
        _LIB = L
    return _LIB


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


def _check(rc):
    if rc != 0:
        raise RuntimeError("reference harness: " + lib().rr_last_error().decode())


class RefHarness:
    def __init__(self, data, eta=-1.0, initial_value=0.001, noise_cut=10.0, threshold=0.0,
                 normalize=False, vis_noise=-1.0):
        L = lib()
        _check(L.rr_load(CUBIN.encode()))
        self.M, self.N = data.M, data.N
        self.freq = np.ascontiguousarray(data.freqs, dtype=np.float32)
        self.chan_off = np.ascontiguousarray(data.chan_off, dtype=np.int64)
        self.uvw = np.ascontiguousarray(data.uvw_m, dtype=np.float64)
        self.vo = np.ascontiguousarray(data.vo, dtype=np.float32)
        self.w = np.ascontiguousarray(data.weight, dtype=np.float32)
        self.minpix = np.float32(initial_value * -1.0 * eta)
        h = C.c_void_p()
        _check(L.rr_create(data.M, data.N, data.DELTAX, data.DELTAY, data.xobs, data.yobs,
                           data.nu_0, data.antenna_diameter, data.pb_factor, data.pb_cutoff,
                           data.primary_beam, vis_noise, noise_cut, eta, initial_value, threshold,
                           int(normalize), len(self.freq), _p(self.freq, C.c_float),
                           _p(self.chan_off, C.c_long), _p(self.uvw, C.c_double),
                           _p(self.vo, C.c_float), _p(self.w, C.c_float), C.byref(h)))
        self.h = h
        fg, nc = C.c_float(), C.c_float()
        self.noise = np.zeros(self.M * self.N, dtype=np.float32)
        _check(L.rr_info(h, C.byref(fg), C.byref(nc), _p(self.noise, C.c_float)))
        self.fg_scale, self.noise_cut = fg.value, nc.value

    def close(self):
        if getattr(self, "h", None):
            lib().rr_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def initial_image(self):
        img = np.zeros((2, self.N, self.M), dtype=np.float32)
        img[0] = self.minpix
        return img

    def chi2(self, img, flag_opt=0):
        img = np.ascontiguousarray(img, dtype=np.float32).copy()
        v = C.c_float()
        _check(lib().rr_chi2(self.h, _p(img, C.c_float), flag_opt, C.byref(v)))
        return v.value, img

    def dchi2(self, img, flag_opt=0):
        img = np.ascontiguousarray(img, dtype=np.float32)
        out = np.zeros((2, self.N, self.M), dtype=np.float32)
        _check(lib().rr_dchi2(self.h, _p(img, C.c_float), flag_opt, _p(out, C.c_float)))
        return out

    def dchi2_band(self, img, i0, rows, flag_opt=0):
        """dchi2() over image rows [i0, i0 + rows) only (multiples of 16):
        both result planes of those rows, (2, rows, N)."""
        img = np.ascontiguousarray(img, dtype=np.float32)
        out = np.zeros((2, rows, self.N), dtype=np.float32)
        _check(lib().rr_dchi2_band(self.h, _p(img, C.c_float), flag_opt, int(i0), int(rows),
                                   _p(out, C.c_float)))
        return out

    def residuals(self):
        out = np.zeros((int(self.chan_off[-1]), 2), dtype=np.float32)
        _check(lib().rr_residuals(self.h, _p(out, C.c_float)))
        return out

    def prior(self, kind, lam, img, G=0.001, eta=-1.0, eps=1e-12, index=0):
        img = np.ascontiguousarray(img, dtype=np.float32)
        v = C.c_float()
        g = np.zeros((self.N, self.M), dtype=np.float32)
        _check(lib().rr_prior(self.h, kind, lam, G, eta, eps, index, _p(img, C.c_float),
                              C.byref(v), _p(g, C.c_float)))
        return v.value, g

    def time(self, img, reps=3, band_rows=256):
        img = np.ascontiguousarray(img, dtype=np.float32)
        a, b = C.c_double(), C.c_double()
        _check(lib().rr_time(self.h, _p(img, C.c_float), reps, band_rows, C.byref(a), C.byref(b)))
        return a.value, b.value
