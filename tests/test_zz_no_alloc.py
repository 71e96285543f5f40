"""gv_prior_value_static: the allocation-free prior value.

Callers such as a plugin running inside a framework that owns every byte of
device memory, or a real-time loop that must not risk an allocation's
implicit device synchronisation, cannot call cudaMalloc.  This entry point
takes all inputs and outputs from the caller and keeps its scratch in a
static device array inside the library.  The test calls it through the C ABI
and checks it against gv_prior_value (which uses the problem's own scratch)
on two calls in a row, within the tolerance of the other prior tests.

The file is named so that pytest collects it last; it also passes when run
alone in a fresh process.
"""

import ctypes as C

import numpy as np
import pytest

from gpuvmem_gb300 import synth

pytestmark = pytest.mark.gpu

PRIORS = [  # kind, lambda, image_index, image_to_add, prior_value, eta, epsilon
    (0, 1.0, 0, 0, 0.0, 0.0, 0.0),
    (1, 0.01, 0, 0, 0.001, -1.0, 0.0),
    (2, 1e-4, 0, 0, 0.0, 0.0, 0.0),
    (3, 1e-4, 0, 0, 0.0, 0.0, 1e-12),
    (4, 1e-3, 0, 0, 0.0, 0.0, 1e-12),
    (5, 1e-5, 0, 0, 0.0, 0.0, 0.0),
]


def test_prior_value_static_matches_problem_entry_point():
    import torch
    import gpuvmem_gb300 as gv

    L = gv.lib()
    fn = L.gv_prior_value_static
    fn.argtypes = [C.c_int32, C.c_void_p, C.c_void_p, C.c_float, C.c_int32, C.c_float,
                   C.c_float, C.c_float, C.c_void_p, C.c_void_p]
    fn.restype = C.c_int

    data = synth.generate(synth.small_config(n=64, nchan=2, seed=3))
    prob = gv.Problem(data, PRIORS)
    rng = np.random.default_rng(5)
    img = np.zeros((2, data.N, data.M), dtype=np.float32)
    img[0] = prob.info.minpix
    img[0] += ((rng.uniform(0, 1, img[0].shape) < 0.2) *
               np.abs(rng.normal(0, 2000.0, img[0].shape))).astype(np.float32)
    d_img = torch.from_numpy(img).cuda()
    noise = prob.noise_image()
    cut = prob.info.noise_cut
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call in range(2):
        for t, (kind, lam, idx, add, G, eta, eps) in enumerate(PRIORS):
            if kind == 0:
                continue
            ref = prob.prior_value(t, d_img)
            out.fill_(-1.0)
            rc = fn(kind, C.c_void_p(d_img[idx].data_ptr()), C.c_void_p(noise.data_ptr()), cut,
                    data.N, G, eta, eps, C.c_void_p(out.data_ptr()), stream)
            assert rc == 0, L.gv_last_error()
            torch.cuda.synchronize()
            got = float(out.item())
            assert abs(got - ref) <= 1e-5 * max(abs(ref), 1e-30), (call, kind, got, ref)


def test_prior_value_static_rejects_oversize_and_bad_kind():
    import gpuvmem_gb300 as gv

    L = gv.lib()
    fn = L.gv_prior_value_static
    fn.argtypes = [C.c_int32, C.c_void_p, C.c_void_p, C.c_float, C.c_int32, C.c_float,
                   C.c_float, C.c_float, C.c_void_p, C.c_void_p]
    fn.restype = C.c_int
    dummy = C.c_void_p(16)
    assert fn(1, dummy, dummy, 1.0, 8193, 0.001, -1.0, 0.0, dummy, None) == 4
    assert b"8192" in L.gv_last_error()
    assert fn(0, dummy, dummy, 1.0, 64, 0.0, 0.0, 0.0, dummy, None) == 1
