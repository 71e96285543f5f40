"""ctypes binding of the CPU oracle (gv_oracle.c).

TEST INFRASTRUCTURE ONLY: tests/, __graft_entry__.smoke() and bench.py's CPU
baseline load this module; the product path never does.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None

OR_AIRYDISK, OR_GAUSSIAN = 0, 1
FI_CHI2, FI_ENTROPY, FI_TSV, FI_TV, FI_L1, FI_LAPLACIAN, FI_GENTROPY, FI_GL1, FI_QUADRATIC = \
    range(9)


class OrTerm(C.Structure):
    _fields_ = [("kind", C.c_int), ("lam", C.c_float), ("image_index", C.c_int),
                ("image_to_add", C.c_int), ("prior_value", C.c_float),
                ("eta", C.c_float), ("epsilon", C.c_float),
                ("prior_image", C.POINTER(C.c_float)), ("epsilon_b", C.c_float)]


class OrProblem(C.Structure):
    _fields_ = [("M", C.c_int), ("N", C.c_int), ("DELTAX", C.c_double),
                ("DELTAY", C.c_double), ("xobs", C.c_float), ("yobs", C.c_float),
                ("nu_0", C.c_float), ("antenna_diameter", C.c_float),
                ("pb_factor", C.c_float), ("pb_cutoff", C.c_float),
                ("primary_beam", C.c_int), ("eta", C.c_float), ("minpix", C.c_float),
                ("threshold", C.c_float), ("noise_cut", C.c_float),
                ("fg_scale", C.c_float), ("normalize", C.c_int), ("nchan", C.c_int),
                ("freq", C.POINTER(C.c_float)), ("chan_off", C.POINTER(C.c_int64)),
                ("uvw", C.POINTER(C.c_double)), ("vo", C.POINTER(C.c_float)),
                ("weight", C.POINTER(C.c_float)), ("noise", C.POINTER(C.c_float)),
                ("nterms", C.c_int), ("terms", C.POINTER(OrTerm)),
                ("gcf", C.POINTER(C.c_float))]


class OrState(C.Structure):
    _fields_ = [("p", C.POINTER(OrProblem)), ("iteration", C.c_int),
                ("flag_opt", C.c_int), ("vr", C.POINTER(C.c_double)),
                ("last_fi", C.c_double * 8), ("nevals", C.c_long), ("ngrads", C.c_long)]


class OrReport(C.Structure):
    _fields_ = [("iterations", C.c_int), ("exit_reason", C.c_int),
                ("f_final", C.c_float), ("nevals", C.c_long), ("ngrads", C.c_long)]


def build():
    """Compile liboracle.so in place (gcc + OpenMP)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = C.CDLL(path)
        f64p, f32p, i64p = C.POINTER(C.c_double), C.POINTER(C.c_float), C.POINTER(C.c_int64)
        L.or_hermitian.argtypes = [C.c_int64, f64p, f32p, C.c_float]
        L.or_noise_and_beam.argtypes = [C.c_int, f32p, i64p, f64p, f32p, f64p, f64p, f64p, f32p]
        L.or_noise_and_beam.restype = C.c_float
        L.or_noise_image.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, C.c_float,
                                     C.c_float, C.c_float, C.c_float, C.c_float, C.c_float,
                                     C.c_int, C.c_double, C.c_double, C.c_float, C.c_float,
                                     f32p, f32p]
        L.or_noise_image.restype = C.c_float
        L.or_attenuation.argtypes = [C.c_int, C.c_int, C.c_float, C.c_float, C.c_double,
                                     C.c_double, C.c_float, C.c_float, C.c_float, C.c_float,
                                     C.c_int]
        L.or_attenuation.restype = C.c_float
        P = C.POINTER(OrProblem)
        L.or_clip.argtypes = [P, f32p, C.c_int]
        L.or_chi2.argtypes = [P, f32p, C.c_int, f64p]
        L.or_chi2.restype = C.c_double
        L.or_model_vis.argtypes = [P, f32p, f64p]
        L.or_dchi2.argtypes = [P, f32p, f64p, C.c_int, f64p]
        L.or_dchi2_channel.argtypes = [P, C.c_int, f64p, f64p]
        L.or_dchi2_pixels.argtypes = [P, C.c_int, f64p, C.c_int, C.POINTER(C.c_int64), f64p]
        L.or_prior_value.argtypes = [P, C.POINTER(OrTerm), f32p]
        L.or_prior_value.restype = C.c_double
        L.or_prior_grad.argtypes = [P, C.POINTER(OrTerm), f32p, f64p]
        S = C.POINTER(OrState)
        L.or_calc_function.argtypes = [S, f32p]
        L.or_calc_function.restype = C.c_double
        L.or_calc_gradient.argtypes = [S, f32p, f32p, C.c_int]
        L.or_frprmn.argtypes = [S, f32p, C.c_int, C.c_float, C.c_float, C.c_int, C.POINTER(OrReport)]
        L.or_lbfgs.argtypes = [S, f32p, C.c_int, C.c_int, C.c_float, C.c_float, C.c_int,
                               C.POINTER(OrReport)]
        L.or_fft2d_inverse.argtypes = [C.c_int, f64p]
        L.or_num_threads.restype = C.c_int
        _LIB = L
    return _LIB


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


def fft2d_inverse(x: np.ndarray) -> np.ndarray:
    n = x.shape[0]
    buf = np.ascontiguousarray(np.stack([x.real, x.imag], axis=-1).astype(np.float64))
    lib().or_fft2d_inverse(n, _p(buf, C.c_double))
    return buf[..., 0] + 1j * buf[..., 1]


class Oracle:
    """Set-up and evaluation of one problem on the CPU, following the
    reference's MFS::setDevice and chi2()/dchi2() order."""

    def __init__(self, data, terms, eta=-1.0, initial_value=0.001, noise_cut=10.0,
                 threshold=0.0, normalize=False, vis_noise=-1.0, gcf=None):
        L = lib()
        self.data = data
        self.M, self.N = data.M, data.N
        self.freqs = np.ascontiguousarray(data.freqs, dtype=np.float32)
        self.chan_off = np.ascontiguousarray(data.chan_off, dtype=np.int64)
        nc = len(self.freqs)
        uvw_m = np.ascontiguousarray(data.uvw_m, dtype=np.float64)
        self.weight = np.ascontiguousarray(data.weight, dtype=np.float32).copy()
        bmaj, bmin, bpa = C.c_double(), C.c_double(), C.c_double()
        vn = C.c_float(vis_noise)
        self.sum_weights = L.or_noise_and_beam(nc, _p(self.freqs, C.c_float),
                                               _p(self.chan_off, C.c_int64),
                                               _p(uvw_m, C.c_double), _p(self.weight, C.c_float),
                                               C.byref(bmaj), C.byref(bmin), C.byref(bpa),
                                               C.byref(vn))
        self.bmaj, self.bmin, self.bpa, self.vis_noise = bmaj.value, bmin.value, bpa.value, vn.value
        self.uvw = uvw_m.copy()
        self.vo = np.ascontiguousarray(data.vo, dtype=np.float32).copy()
        for c in range(nc):
            o, e = self.chan_off[c], self.chan_off[c + 1]
            u = np.ascontiguousarray(self.uvw[o:e])
            v = np.ascontiguousarray(self.vo[o:e])
            L.or_hermitian(e - o, _p(u, C.c_double), _p(v, C.c_float), C.c_float(self.freqs[c]))
            self.uvw[o:e] = u
            self.vo[o:e] = v
        self.noise = np.zeros(self.M * self.N, dtype=np.float32)
        cut = C.c_float()
        self.fg_scale = L.or_noise_image(self.M, self.N, data.DELTAX, data.DELTAY, data.xobs,
                                         data.yobs, data.nu_0, data.antenna_diameter,
                                         data.pb_factor, data.pb_cutoff, data.primary_beam,
                                         self.bmaj, self.bmin, self.vis_noise, noise_cut,
                                         _p(self.noise, C.c_float), C.byref(cut))
        self.noise_cut = cut.value
        self.minpix = np.float32(initial_value * -1.0 * eta)
        self.terms_list = list(terms)
        self.terms = (OrTerm * max(1, len(terms)))()
        for i, t in enumerate(terms):
            self.terms[i] = OrTerm(*t[:7])
            if len(t) > 7:
                # GEntropy / GL1Norm: the prior image divided by its factor
                # in FP32, as normalizePrior does
                pr = (np.asarray(t[7], np.float32).reshape(-1) /
                      np.float32(t[8] if t[8] else 1.0)).astype(np.float32)
                self._priors = getattr(self, "_priors", []) + [pr]
                self.terms[i].prior_image = _p(pr, C.c_float)
                self.terms[i].epsilon_b = float(t[9])
        self.prob = OrProblem(
            self.M, self.N, data.DELTAX, data.DELTAY, data.xobs, data.yobs, data.nu_0,
            data.antenna_diameter, data.pb_factor, data.pb_cutoff, data.primary_beam,
            eta, float(self.minpix), threshold, self.noise_cut, self.fg_scale, int(normalize),
            nc, _p(self.freqs, C.c_float), _p(self.chan_off, C.c_int64),
            _p(self.uvw, C.c_double), _p(self.vo, C.c_float), _p(self.weight, C.c_float),
            _p(self.noise, C.c_float), len(terms), self.terms)
        # gridding correction function of gridded data (apply_GCF / GCF DChi2)
        self.gcf = None if gcf is None else np.ascontiguousarray(gcf, np.float32).reshape(-1)
        if self.gcf is not None:
            self.prob.gcf = _p(self.gcf, C.c_float)
        self.vr = np.zeros(2 * self.chan_off[-1], dtype=np.float64)
        self.state = OrState(C.pointer(self.prob), 0, 0, _p(self.vr, C.c_double),
                             (C.c_double * 8)(), 0, 0)

    @property
    def mask(self):
        return (self.noise < self.noise_cut).reshape(self.N, self.M)

    def initial_image(self):
        img = np.zeros((2, self.N, self.M), dtype=np.float32)
        img[0] = self.minpix
        return img

    def chi2(self, img, flag_opt=0):
        img = np.ascontiguousarray(img, dtype=np.float32)
        v = lib().or_chi2(C.byref(self.prob), _p(img, C.c_float), flag_opt, _p(self.vr, C.c_double))
        return v, img

    def model_vis(self, img):
        img = np.ascontiguousarray(img, dtype=np.float32)
        vm = np.zeros(2 * self.chan_off[-1], dtype=np.float64)
        lib().or_model_vis(C.byref(self.prob), _p(img, C.c_float), _p(vm, C.c_double))
        return vm.reshape(-1, 2)

    def dchi2(self, img, flag_opt=0):
        img = np.ascontiguousarray(img, dtype=np.float32)
        out = np.zeros(2 * self.M * self.N, dtype=np.float64)
        lib().or_dchi2(C.byref(self.prob), _p(img, C.c_float), _p(self.vr, C.c_double),
                       flag_opt, _p(out, C.c_double))
        return out.reshape(2, self.N, self.M)

    def dchi2_channel(self, c):
        out = np.zeros(self.M * self.N, dtype=np.float64)
        lib().or_dchi2_channel(C.byref(self.prob), c, _p(self.vr, C.c_double), _p(out, C.c_double))
        return out.reshape(self.N, self.M)

    def dchi2_pixels(self, c, pix):
        pix = np.ascontiguousarray(pix, dtype=np.int64)
        out = np.zeros(pix.size, dtype=np.float64)
        lib().or_dchi2_pixels(C.byref(self.prob), c, _p(self.vr, C.c_double), pix.size,
                              _p(pix, C.c_int64), _p(out, C.c_double))
        return out

    def prior_value(self, ti, img):
        img = np.ascontiguousarray(img, dtype=np.float32)
        return lib().or_prior_value(C.byref(self.prob), C.byref(self.terms[ti]), _p(img, C.c_float))

    def prior_grad(self, ti, img):
        img = np.ascontiguousarray(img, dtype=np.float32)
        out = np.zeros(self.M * self.N, dtype=np.float64)
        lib().or_prior_grad(C.byref(self.prob), C.byref(self.terms[ti]), _p(img, C.c_float),
                            _p(out, C.c_double))
        return out.reshape(self.N, self.M)

    def calc_function(self, img, flag_opt=0):
        self.state.flag_opt = flag_opt
        img = np.ascontiguousarray(img, dtype=np.float32)
        v = lib().or_calc_function(C.byref(self.state), _p(img, C.c_float))
        return v, img

    def calc_gradient(self, img, it, flag_opt=0):
        self.state.flag_opt = flag_opt
        img = np.ascontiguousarray(img, dtype=np.float32)
        xi = np.zeros_like(img)
        lib().or_calc_gradient(C.byref(self.state), _p(img, C.c_float), _p(xi, C.c_float), it)
        return xi

    def optimize(self, img, method="frprmn", iterations=10, ftol=1e-12, gtol=1e-12, K=100,
                 positivity=True, flag_opt=0):
        self.state.flag_opt = flag_opt
        self.state.iteration = 0
        img = np.ascontiguousarray(img, dtype=np.float32).copy()
        rep = OrReport()
        if method == "frprmn":
            lib().or_frprmn(C.byref(self.state), _p(img, C.c_float), iterations, ftol, gtol,
                            int(positivity), C.byref(rep))
        else:
            lib().or_lbfgs(C.byref(self.state), _p(img, C.c_float), iterations, K, ftol, gtol,
                           int(positivity), C.byref(rep))
        return img, rep
