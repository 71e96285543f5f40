"""gpuvmem_gb300: GB300-native imaging-objective path of gpuvmem.

Python view of the C ABI in include/gpuvmem_gb300.h (ctypes).  Device
buffers are torch CUDA tensors; torch is used for device memory and streams
only -- every computation runs in the in-tree CUDA library
libgpuvmem_gb300.so.  There is no CPU fallback: if the library is missing
the import of `lib()` raises.
"""

from __future__ import annotations

import ctypes as C
import os
from typing import Optional, Sequence

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libgpuvmem_gb300.so")
_LIB = None

GV_OK = 0
STATUS = {0: "GV_OK", 1: "GV_ERR_INVALID", 2: "GV_ERR_CUDA", 3: "GV_ERR_NOMEM",
          4: "GV_ERR_UNSUPPORTED", 5: "GV_ERR_DEVICE"}
FI_CHI2, FI_ENTROPY, FI_TSV, FI_TV, FI_L1, FI_LAPLACIAN, FI_GENTROPY, FI_GL1, FI_QUADRATIC = \
    range(9)
FI_IDS = {"Chi2": FI_CHI2, "Entropy": FI_ENTROPY, "TotalSquaredVariation": FI_TSV,
          "TotalVariation": FI_TV, "L1-Norm": FI_L1, "Laplacian": FI_LAPLACIAN,
          "GEntropy": FI_GENTROPY, "GL1Norm": FI_GL1, "Quadratic": FI_QUADRATIC}
OPT_FRPRMN, OPT_LBFGS = 0, 1
OPT_IDS = {"CG-FRPRMN": OPT_FRPRMN, "CG-LBFGS": OPT_LBFGS}


class GvError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class FiDesc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("lam", C.c_float), ("image_index", C.c_int32),
                ("image_to_add", C.c_int32), ("prior_value", C.c_float), ("eta", C.c_float),
                ("epsilon", C.c_float), ("prior_image", C.POINTER(C.c_float)),
                ("normalization_factor", C.c_float), ("epsilon_b", C.c_float)]


class ChannelDesc(C.Structure):
    _fields_ = [("freq_hz", C.c_float), ("nvis", C.c_int64), ("uvw", C.POINTER(C.c_double)),
                ("vo", C.POINTER(C.c_float)), ("weight", C.POINTER(C.c_float))]


class ProblemDesc(C.Structure):
    _fields_ = [("M", C.c_int32), ("N", C.c_int32), ("deltax_deg", C.c_double),
                ("deltay_deg", C.c_double), ("xobs_pix", C.c_float), ("yobs_pix", C.c_float),
                ("nu_0", C.c_float), ("antenna_diameter", C.c_float), ("pb_factor", C.c_float),
                ("pb_cutoff", C.c_float), ("primary_beam", C.c_int32), ("vis_noise", C.c_float),
                ("noise_cut_factor", C.c_float), ("eta", C.c_float),
                ("initial_value", C.c_float), ("threshold", C.c_float),
                ("normalize", C.c_int32), ("nchannels", C.c_int32),
                ("channels", C.POINTER(ChannelDesc)), ("nterms", C.c_int32),
                ("terms", C.POINTER(FiDesc)), ("dchi2_engine", C.c_int32),
                ("gcf", C.POINTER(C.c_float))]


class CKernelDesc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("m", C.c_int32), ("n", C.c_int32), ("amp", C.c_float),
                ("w", C.c_float), ("alpha", C.c_float), ("w2", C.c_float)]


class GridKernel(C.Structure):
    _fields_ = [("m", C.c_int32), ("n", C.c_int32), ("support_x", C.c_int32),
                ("support_y", C.c_int32), ("values", C.POINTER(C.c_float))]


class ProblemInfo(C.Structure):
    _fields_ = [("fg_scale", C.c_float), ("noise_cut", C.c_float), ("vis_noise", C.c_float),
                ("minpix", C.c_float), ("beam_bmaj_deg", C.c_double),
                ("beam_bmin_deg", C.c_double), ("beam_bpa_deg", C.c_double),
                ("sum_weights", C.c_float), ("nvis_total", C.c_int64),
                ("nvis_in_grid", C.c_int64), ("mask_pixels", C.c_int64),
                ("dchi2_engine", C.c_int32), ("nterms", C.c_int32)]


class OptDesc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("total_iterations", C.c_int32), ("ftol", C.c_float),
                ("gtol", C.c_float), ("K", C.c_int32), ("flag", C.c_int32),
                ("positivity", C.c_int32)]


class TuneReport(C.Structure):
    _fields_ = [("tc_pair", C.c_int32), ("tc_nsplit", C.c_int32), ("degrid_threads", C.c_int32),
                ("degrid_blocks", C.c_int32), ("dchi2_ms_default", C.c_double),
                ("dchi2_ms_tuned", C.c_double), ("chi2_ms_default", C.c_double),
                ("chi2_ms_tuned", C.c_double), ("candidates", C.c_int32)]


class OptReport(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("exit_reason", C.c_int32), ("f_final", C.c_float),
                ("n_objective", C.c_int64), ("n_gradient", C.c_int64), ("seconds", C.c_double)]


EXPORTS = ["gv_problem_create", "gv_problem_destroy", "gv_problem_info_get",
           "gv_problem_set_stream", "gv_noise_image", "gv_initial_image", "gv_chi2", "gv_dchi2",
           "gv_dchi2_channel", "gv_prior_value", "gv_prior_gradient", "gv_objective",
           "gv_gradient", "gv_optimize", "gv_dirty_image", "gv_residuals", "gv_last_error",
           "gv_version", "gv_launch_count"]


def lib():
    """Load libgpuvmem_gb300.so; raises if it was not built."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: run __graft_entry__.build() "
                          "(python -m gpuvmem_gb300.build)")
    L = C.CDLL(LIB_PATH)
    vp, i32, i64, f32, f64 = C.c_void_p, C.c_int32, C.c_int64, C.c_float, C.c_double
    f64p, f32p = C.POINTER(C.c_double), C.POINTER(C.c_float)
    sig = {
        "gv_problem_create": [C.POINTER(ProblemDesc), C.POINTER(vp)],
        "gv_problem_destroy": [vp],
        "gv_problem_info_get": [vp, C.POINTER(ProblemInfo)],
        "gv_problem_set_stream": [vp, vp],
        "gv_noise_image": [vp, vp],
        "gv_initial_image": [vp, vp],
        "gv_chi2": [vp, vp, i32, f64p],
        "gv_dchi2": [vp, vp, i32, vp],
        "gv_dchi2_channel": [vp, i32, vp],
        "gv_prior_value": [vp, i32, vp, f64p],
        "gv_prior_gradient": [vp, i32, vp, vp],
        "gv_objective": [vp, vp, i32, f64p, f64p],
        "gv_objective_many": [vp, C.POINTER(vp), i32, i32, f64p, f64p],
        "gv_gradient": [vp, vp, vp, i32, i32],
        "gv_evaluate": [vp, vp, vp, i32, i32, f64p, f64p],
        "gv_problem_set_graphs": [vp, i32],
        "gv_optimize": [vp, C.POINTER(OptDesc), vp, C.POINTER(OptReport)],
        "gv_optimize_until": [vp, C.POINTER(OptDesc), vp, f64, i32, C.POINTER(OptReport)],
        "gv_set_iteration": [vp, i32],
        "gv_linmin": [vp, vp, vp, i32, i32, C.POINTER(C.c_float), C.POINTER(C.c_int64)],
        "gv_dirty_image": [vp, vp],
        "gv_psf_image": [vp, vp],
        "gv_residuals": [vp, f32p],
        "gv_autotune": [vp, C.POINTER(TuneReport)],
        "gv_error_images": [vp, vp, vp],
        "gv_apply_weighting": [i32, f32, i32, i32, f64, f64, i32, C.POINTER(ChannelDesc),
                               C.POINTER(C.c_void_p), vp],
        "gv_ckernel_defaults": [i32, i32, i32, C.POINTER(CKernelDesc)],
        "gv_ckernel_build": [C.POINTER(CKernelDesc), i32, i32, f64, f64, vp,
                             C.POINTER(i32), C.POINTER(i32), vp, C.POINTER(i32)],
        "gv_grid_visibilities": [C.POINTER(GridKernel), i32, i32, f64, f64, i32,
                                 C.POINTER(ChannelDesc), C.POINTER(ChannelDesc), vp],
        "gv_batch_create": [C.POINTER(vp), i32, C.POINTER(vp)],
        "gv_batch_destroy": [vp],
        "gv_batch_set_graphs": [vp, i32],
        "gv_batch_evaluate": [vp, C.POINTER(vp), C.POINTER(vp), i32, i32, f64p],
    }
    for name, args in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = C.c_int
    L.gv_launch_count.restype = C.c_int64
    L.gv_last_error.restype = C.c_char_p
    L.gv_version.restype = C.c_char_p
    _LIB = L
    return L


def launch_count() -> int:
    """Kernels launched by the library so far in this process."""
    return int(lib().gv_launch_count())


def check(status):
    if status != GV_OK:
        raise GvError(status, lib().gv_last_error().decode())


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def term(kind, lam, image_index=0, image_to_add=0, prior_value=0.001, eta=-1.0, epsilon=1e-12,
         prior_image=None, normalization_factor=1.0, epsilon_b=1e-12):
    """One ObjectiveFunction term, as Fi::configure + setPrior would set it;
    GEntropy and GL1Norm take a prior image (M*N) and its normalisation
    factor, GL1Norm also epsilon_b (epsilon is its epsilon_a)."""
    if isinstance(kind, str):
        kind = FI_IDS[kind]
    t = (int(kind), float(lam), int(image_index), int(image_to_add), float(prior_value),
         float(eta), float(epsilon))
    if prior_image is not None:
        t += (np.ascontiguousarray(prior_image, dtype=np.float32).reshape(-1),
              float(normalization_factor), float(epsilon_b))
    return t


def _fi_desc(t, keep):
    """FiDesc of a term tuple (7 fields, or 10 with a prior image)."""
    d = FiDesc(*t[:7])
    if len(t) > 7:
        img = np.ascontiguousarray(t[7], dtype=np.float32).reshape(-1)
        keep.append(img)
        d.prior_image = img.ctypes.data_as(C.POINTER(C.c_float))
        d.normalization_factor = float(t[8])
        d.epsilon_b = float(t[9])
    else:
        d.normalization_factor = 1.0
        d.epsilon_b = 1e-12
    return d


class Problem:
    """One imaging problem resident on the current CUDA device."""

    def __init__(self, data, terms: Sequence[tuple], eta=-1.0, initial_value=0.001,
                 noise_cut=10.0, threshold=0.0, normalize=False, engine=0, vis_noise=-1.0,
                 stream=None, gcf=None):
        L = lib()
        self.data = data
        self.M, self.N = data.M, data.N
        C_ = len(data.freqs)
        self._keep = []
        chans = (ChannelDesc * C_)()
        for c in range(C_):
            o, e = int(data.chan_off[c]), int(data.chan_off[c + 1])
            uvw = np.ascontiguousarray(data.uvw_m[o:e], dtype=np.float64)
            vo = np.ascontiguousarray(data.vo[o:e], dtype=np.float32)
            w = np.ascontiguousarray(data.weight[o:e], dtype=np.float32)
            self._keep += [uvw, vo, w]
            chans[c] = ChannelDesc(float(data.freqs[c]), e - o,
                                   uvw.ctypes.data_as(C.POINTER(C.c_double)),
                                   vo.ctypes.data_as(C.POINTER(C.c_float)),
                                   w.ctypes.data_as(C.POINTER(C.c_float)))
        tl = (FiDesc * max(1, len(terms)))()
        for i, t in enumerate(terms):
            tl[i] = _fi_desc(t, self._keep)
        self.terms = [t for t in terms if t[1] != 0.0]
        desc = ProblemDesc(data.M, data.N, data.DELTAX, data.DELTAY, data.xobs, data.yobs,
                           data.nu_0, data.antenna_diameter, data.pb_factor, data.pb_cutoff,
                           data.primary_beam, vis_noise, noise_cut, eta, initial_value,
                           threshold, int(normalize), C_, chans, len(terms), tl, engine)
        if gcf is not None:
            # gridding correction function of gridded data (Chi2::setCKernel)
            g = np.ascontiguousarray(gcf, dtype=np.float32).reshape(-1)
            if g.size != self.M * self.N:
                raise ValueError("gcf must have M*N values")
            self._keep.append(g)
            desc.gcf = g.ctypes.data_as(C.POINTER(C.c_float))
        h = C.c_void_p()
        check(L.gv_problem_create(C.byref(desc), C.byref(h)))
        self.h = h
        import torch
        # the device the problem's buffers live on (the current one)
        self.device = torch.device("cuda", torch.cuda.current_device())
        if stream is not None:
            self.set_stream(stream)

    def close(self):
        if getattr(self, "h", None):
            lib().gv_problem_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream):
        check(lib().gv_problem_set_stream(self.h, C.c_void_p(stream)))

    @property
    def info(self) -> ProblemInfo:
        inf = ProblemInfo()
        check(lib().gv_problem_info_get(self.h, C.byref(inf)))
        return inf

    def _img(self):
        import torch
        return torch.zeros((2, self.N, self.M), dtype=torch.float32, device="cuda")

    def initial_image(self):
        img = self._img()
        check(lib().gv_initial_image(self.h, _ptr(img)))
        return img

    def noise_image(self):
        import torch
        out = torch.empty((self.N, self.M), dtype=torch.float32, device="cuda")
        check(lib().gv_noise_image(self.h, _ptr(out)))
        return out

    def chi2(self, img, flag_opt=0) -> float:
        v = C.c_double()
        check(lib().gv_chi2(self.h, _ptr(img), flag_opt, C.byref(v)))
        return v.value

    def dchi2(self, img, flag_opt=0, out=None):
        if out is None:
            out = self._img()
        check(lib().gv_dchi2(self.h, _ptr(img), flag_opt, _ptr(out)))
        return out

    def dchi2_channel(self, c):
        import torch
        out = torch.zeros((self.N, self.M), dtype=torch.float32, device="cuda")
        check(lib().gv_dchi2_channel(self.h, c, _ptr(out)))
        return out

    def prior_value(self, t, img) -> float:
        v = C.c_double()
        check(lib().gv_prior_value(self.h, t, _ptr(img), C.byref(v)))
        return v.value

    def prior_gradient(self, t, img, dphi=None):
        if dphi is None:
            dphi = self._img()
        check(lib().gv_prior_gradient(self.h, t, _ptr(img), _ptr(dphi)))
        return dphi

    def objective(self, img, flag_opt=0):
        f = C.c_double()
        fi = (C.c_double * 8)()
        check(lib().gv_objective(self.h, _ptr(img), flag_opt, C.byref(f), fi))
        return f.value, list(fi)[:len(self.terms)]

    def objective_many(self, imgs, flag_opt=0):
        """objective() of every image in imgs ([n, 2, N, M] or a list of
        [2, N, M]) with one synchronisation; the images are not clipped.
        Returns the n values of f."""
        import torch
        n = len(imgs)
        for i in range(n):
            t = imgs[i]
            if (t.dtype != torch.float32 or not t.is_cuda or not t.is_contiguous()
                    or t.numel() != 2 * self.N * self.M):
                raise ValueError(f"image {i}: need a contiguous float32 CUDA tensor of "
                                 f"2 x {self.N} x {self.M} values")
            if t.device != self.device:
                raise ValueError(f"image {i} is on {t.device}, the problem on {self.device}")
        ptrs = (C.c_void_p * n)(*[imgs[i].data_ptr() for i in range(n)])
        f = (C.c_double * max(n, 1))()
        check(lib().gv_objective_many(self.h, ptrs, n, flag_opt, f, None))
        return [f[i] for i in range(n)]

    def gradient(self, img, it, flag_opt=0, xi=None):
        if xi is None:
            xi = self._img()
        check(lib().gv_gradient(self.h, _ptr(img), _ptr(xi), it, flag_opt))
        return xi

    def evaluate(self, img, it, flag_opt=0, xi=None):
        """objective() then gradient() in one call, replayed from a CUDA graph
        after the first call with the same buffers; returns (f, fi, xi)."""
        if xi is None:
            xi = self._img()
        f = C.c_double()
        fi = (C.c_double * 8)()
        check(lib().gv_evaluate(self.h, _ptr(img), _ptr(xi), it, flag_opt, C.byref(f), fi))
        return f.value, list(fi)[:len(self.terms)], xi

    def set_graphs(self, enable: bool):
        """Replay the optimiser's objective evaluations from CUDA graphs."""
        check(lib().gv_problem_set_graphs(self.h, int(bool(enable))))

    def optimize(self, img, method="CG-FRPRMN", iterations=10, ftol=1e-12, gtol=1e-12, K=100,
                 flag=0, positivity=True) -> OptReport:
        kind = OPT_IDS[method] if isinstance(method, str) else method
        o = OptDesc(kind, iterations, ftol, gtol, K, flag, int(positivity))
        rep = OptReport()
        check(lib().gv_optimize(self.h, C.byref(o), _ptr(img), C.byref(rep)))
        return rep

    def mfs_run(self, img, method="CG-FRPRMN", iterations=10, ftol=1e-12, gtol=1e-12, K=100,
                flags=(0, 1, 2, 3), positivity=True):
        """MFS::run for a two-image fit without an Order (src/mfs.cu:999-1008):
        the optimiser runs once per flag, 0 (I_nu0), 1 (alpha), 2 (I_nu0 with
        the alpha clip below threshold), 3 (alpha), each from the image the
        previous one left.  Returns the reports."""
        return [self.optimize(img, method, iterations=iterations, ftol=ftol, gtol=gtol, K=K,
                              flag=f, positivity=positivity) for f in flags]

    def optimize_until(self, img, f_target, method="CG-FRPRMN", iterations=10, ftol=1e-12,
                       gtol=1e-12, K=100, flag=0, positivity=True,
                       priors_from_start=False) -> OptReport:
        """optimize(), also stopping once f <= f_target (exit_reason 4)."""
        kind = OPT_IDS[method] if isinstance(method, str) else method
        o = OptDesc(kind, iterations, ftol, gtol, K, flag, int(positivity))
        rep = OptReport()
        check(lib().gv_optimize_until(self.h, C.byref(o), _ptr(img), float(f_target),
                                      int(bool(priors_from_start)), C.byref(rep)))
        return rep

    def linmin(self, p, xi, flag_opt=0, positivity=True):
        """linmin (src/linmin.cu:52-110): minimise the objective along xi
        from p; p and xi are updated in place as newP leaves them.  Returns
        (fret, objective evaluations)."""
        fret = C.c_float()
        evals = C.c_int64()
        check(lib().gv_linmin(self.h, _ptr(p), _ptr(xi), flag_opt, int(bool(positivity)),
                              C.byref(fret), C.byref(evals)))
        return fret.value, evals.value

    def error_images(self, img):
        """calculateErrors: (2, N, M) error images of the solution img."""
        out = self._img()
        check(lib().gv_error_images(self.h, _ptr(img), _ptr(out)))
        return out

    def autotune(self) -> TuneReport:
        """Measure and keep the fastest DChi2 and degridding launch shapes."""
        r = TuneReport()
        check(lib().gv_autotune(self.h, C.byref(r)))
        return r

    def set_iteration(self, it: int):
        check(lib().gv_set_iteration(self.h, int(it)))

    def dirty_image(self):
        import torch
        out = torch.zeros((self.N, self.M), dtype=torch.float32, device="cuda")
        check(lib().gv_dirty_image(self.h, _ptr(out)))
        return out

    def psf_image(self):
        import torch
        out = torch.zeros((self.N, self.M), dtype=torch.float32, device="cuda")
        check(lib().gv_psf_image(self.h, _ptr(out)))
        return out

    def residuals(self) -> np.ndarray:
        out = np.zeros((int(self.info.nvis_total), 2), dtype=np.float32)
        check(lib().gv_residuals(self.h, out.ctypes.data_as(C.POINTER(C.c_float))))
        return out


class Batch:
    """gv_batch: one objective + gradient evaluation of several independent
    problems in one CUDA-graph launch."""

    def __init__(self, problems: Sequence["Problem"]):
        self.problems = list(problems)
        arr = (C.c_void_p * len(self.problems))(*[p.h for p in self.problems])
        h = C.c_void_p()
        check(lib().gv_batch_create(arr, len(self.problems), C.byref(h)))
        self.h = h

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            try:
                lib().gv_batch_destroy(h)
            except Exception:
                pass
            self.h = None

    def set_graphs(self, enable: bool):
        check(lib().gv_batch_set_graphs(self.h, int(bool(enable))))

    def evaluate(self, imgs, xis, it, flag_opt=0):
        n = len(self.problems)
        ia = (C.c_void_p * n)(*[t.data_ptr() for t in imgs])
        xa = (C.c_void_p * n)(*[t.data_ptr() for t in xis])
        f = (C.c_double * n)()
        check(lib().gv_batch_evaluate(self.h, ia, xa, it, flag_opt, f))
        return list(f)


WEIGHTING = {"natural": 0, "uniform": 1, "briggs": 2}


def apply_weighting(scheme, robust, M, N, deltax_deg, deltay_deg, freqs, chan_off, uvw_m,
                    weight) -> np.ndarray:
    """WeightingScheme::apply ("Natural", "Uniform", "Briggs") on the GPU for
    one field and one correlation; returns the new float32 weights."""
    C_ = len(freqs)
    uvw_m = np.ascontiguousarray(uvw_m, dtype=np.float64)
    w_in = np.ascontiguousarray(weight, dtype=np.float32)
    out = np.empty_like(w_in)
    chans = (ChannelDesc * C_)()
    outs = (C.c_void_p * C_)()
    for c in range(C_):
        o, e = int(chan_off[c]), int(chan_off[c + 1])
        chans[c].freq_hz = float(np.float32(freqs[c]))
        chans[c].nvis = e - o
        chans[c].uvw = uvw_m[o:e].ctypes.data_as(C.POINTER(C.c_double))
        chans[c].vo = None
        chans[c].weight = w_in[o:e].ctypes.data_as(C.POINTER(C.c_float))
        outs[c] = out[o:e].ctypes.data
    check(lib().gv_apply_weighting(WEIGHTING[scheme], float(robust), int(M), int(N),
                                   float(deltax_deg), float(deltay_deg), C_, chans, outs, None))
    return out


CKERNELS = {"PillBox2D": 0, "Gaussian2D": 1, "Sinc2D": 2, "GaussianSinc2D": 3, "PSWF": 4,
            "pillbox": 0, "gaussian": 1, "sinc": 2, "gaussian_sinc": 3, "pswf": 4}


def ckernel_build(kind, M, N, deltax_deg, deltay_deg, m=None, n=None, **params):
    """MFS::configure's kernel set-up for CKernel `kind` (the reference's
    registration ids or their lower-case names): returns (table [m, n] f32,
    (support_x, support_y), gcf [M, N] f32 or None).  m, n default to the
    reference's constructors: PillBox2D() is 1 x 1, the others 7 x 7;
    params override amp, w, alpha, w2."""
    k = CKERNELS[kind]
    if m is None:
        m = n = 1 if k == 0 else 7
    n = m if n is None else n
    d = CKernelDesc()
    check(lib().gv_ckernel_defaults(k, int(m), int(n), C.byref(d)))
    for key, v in params.items():
        setattr(d, key, float(v))
    table = np.zeros((m, n), np.float32)
    gcf = np.zeros((M, N), np.float32)
    sx, sy, hg = C.c_int32(), C.c_int32(), C.c_int32()
    check(lib().gv_ckernel_build(C.byref(d), int(M), int(N), float(deltax_deg),
                                 float(deltay_deg), table.ctypes.data, C.byref(sx), C.byref(sy),
                                 gcf.ctypes.data, C.byref(hg)))
    return table, (sx.value, sy.value), (gcf if hg.value else None)


def grid_visibilities(table, support, M, N, deltax_deg, deltay_deg, freqs, chan_off, uvw_m, vo,
                      weight):
    """do_gridding on the GPU: returns (chan_off, uvw_m [k, 3] f64, vo [k, 2]
    f32, weight [k] f32) of the gridded visibilities, channel by channel."""
    table = np.ascontiguousarray(table, dtype=np.float32)
    kern = GridKernel(table.shape[0], table.shape[1], int(support[0]), int(support[1]),
                      table.ctypes.data_as(C.POINTER(C.c_float)))
    C_ = len(freqs)
    uvw_m = np.ascontiguousarray(uvw_m, dtype=np.float64)
    vo = np.ascontiguousarray(vo, dtype=np.float32).reshape(-1, 2)
    w = np.ascontiguousarray(weight, dtype=np.float32)
    MN = int(M) * int(N)
    ins, outs = (ChannelDesc * C_)(), (ChannelDesc * C_)()
    bufs = []
    for c in range(C_):
        o, e = int(chan_off[c]), int(chan_off[c + 1])
        ins[c] = ChannelDesc(float(np.float32(freqs[c])), e - o,
                             uvw_m[o:e].ctypes.data_as(C.POINTER(C.c_double)),
                             vo[o:e].ctypes.data_as(C.POINTER(C.c_float)),
                             w[o:e].ctypes.data_as(C.POINTER(C.c_float)))
        ou, ov, ow = np.zeros((MN, 3)), np.zeros((MN, 2), np.float32), np.zeros(MN, np.float32)
        bufs.append((ou, ov, ow))
        outs[c] = ChannelDesc(0.0, 0, ou.ctypes.data_as(C.POINTER(C.c_double)),
                              ov.ctypes.data_as(C.POINTER(C.c_float)),
                              ow.ctypes.data_as(C.POINTER(C.c_float)))
    check(lib().gv_grid_visibilities(C.byref(kern), int(M), int(N), float(deltax_deg),
                                     float(deltay_deg), C_, ins, outs, None))
    counts = [int(outs[c].nvis) for c in range(C_)]
    off = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    return (off, np.concatenate([b[0][:k] for b, k in zip(bufs, counts)]),
            np.concatenate([b[1][:k] for b, k in zip(bufs, counts)]),
            np.concatenate([b[2][:k] for b, k in zip(bufs, counts)]))


def grid(data, kind="PillBox2D", m=None, n=None, **params):
    """The reference's gridding step for a synthetic data set (after its
    weighting scheme): returns (gridded data, gcf) -- pass gcf to Problem."""
    import dataclasses
    table, sup, gcf = ckernel_build(kind, data.M, data.N, data.DELTAX, data.DELTAY, m, n,
                                    **params)
    off, uvw, vo, w = grid_visibilities(table, sup, data.M, data.N, data.DELTAX, data.DELTAY,
                                        data.freqs, data.chan_off, data.uvw_m, data.vo,
                                        data.weight)
    return dataclasses.replace(data, chan_off=off, uvw_m=uvw, vo=vo, weight=w), gcf


def _fp_tolerance(x1, x0):
    """tolFunction (src/fixedpoint.cu:3-18): the largest relative change
    |x1[i] - x0[i]| / |x0[i]| over the entries after the first (0 where x0[i]
    is 0), in FP32."""
    tol = [np.float32(0.0) if np.float32(abs(np.float32(x0[i]))) == 0.0 else
           np.float32(abs(np.float32(x1[i]) - np.float32(x0[i]))) /
           np.float32(abs(np.float32(x0[i]))) for i in range(1, len(x1))]
    return float(max(tol)) if tol else 0.0


def fixed_point_opt(guess, optf, tol, iterations):
    """fixedPointOpt (src/fixedpoint.cu:32-57): iterates x1 = optf(x0) until
    the relative change is at most `tol`, `iterations` are done or an entry
    after the first reaches 1.  Kept as the reference runs it: the start point
    is reused for the first two calls (x0 advances from the third on), and the
    first tolerance is taken against a zero vector.  `optf` maps a list of
    floats (e.g. penalization factors) to a list of floats; it typically
    solves a problem with them."""
    x0 = [float(v) for v in guess]
    x1 = [0.0] * len(x0)
    it = 0
    c_tol = _fp_tolerance(x1, x0)
    while it < iterations and c_tol > tol:
        if it > 1:
            x0 = x1
        x1 = [float(np.float32(v)) for v in optf(list(x0))]
        c_tol = _fp_tolerance(x1, x0)
        if any(v >= 1.0 for v in x1[1:]):
            break
        it += 1
    return x1
