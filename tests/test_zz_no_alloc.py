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


def _fn():
    import gpuvmem_gb300 as gv
    L = gv.lib()
    fn = L.gv_prior_value_static
    fn.argtypes = [C.c_int32, C.c_void_p, C.c_void_p, C.c_float, C.c_int32, C.c_float,
                   C.c_float, C.c_float, C.c_void_p, C.c_void_p]
    fn.restype = C.c_int
    return L, fn


def test_prior_value_static_512_rows():
    """512 columns: each of the 256 threads of a row covers two columns."""
    import torch
    import gpuvmem_gb300 as gv
    L, fn = _fn()
    data = synth.generate(synth.small_config(n=512, n_ant=10, n_times=48, nchan=1, seed=9))
    terms = [PRIORS[0], PRIORS[1], PRIORS[2], PRIORS[5]]
    prob = gv.Problem(data, terms)
    rng = np.random.default_rng(6)
    img = np.zeros((2, data.N, data.M), dtype=np.float32)
    img[0] = prob.info.minpix
    img[0] += ((rng.uniform(0, 1, img[0].shape) < 0.2) *
               np.abs(rng.normal(0, 2000.0, img[0].shape))).astype(np.float32)
    d_img = torch.from_numpy(img).cuda()
    noise = prob.noise_image()
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call in range(2):
        for t, (kind, lam, idx, add, G, eta, eps) in enumerate(terms):
            if kind == 0:
                continue
            ref = prob.prior_value(t, d_img)
            out.fill_(-1.0)
            rc = fn(kind, C.c_void_p(d_img[idx].data_ptr()), C.c_void_p(noise.data_ptr()),
                    prob.info.noise_cut, data.N, G, eta, eps, C.c_void_p(out.data_ptr()), stream)
            assert rc == 0, L.gv_last_error()
            torch.cuda.synchronize()
            got = float(out.item())
            assert abs(got - ref) <= 1e-5 * max(abs(ref), 1e-30), (call, kind, got, ref)
    prob.close()


def test_prior_value_static_at_the_8192_row_limit():
    """The largest image the static scratch takes (8192 rows): TSV and
    entropy values against FP64 sums of the per-pixel FP32 values."""
    import torch
    L, fn = _fn()
    n = 8192
    rng = np.random.default_rng(8)
    plane = (0.001 + (rng.uniform(0, 1, (n, n)) < 0.1) *
             np.abs(rng.normal(0, 5.0, (n, n)))).astype(np.float32)
    noise = np.ones((n, n), dtype=np.float32)
    noise[: n // 8] = 3.0  # outside the mask (noise >= cut)
    cut = np.float32(2.0)
    m = noise < cut
    # TSV, calculateTSV (src/functions.cu:3353): border pixels contribute c
    dx = np.zeros_like(plane)
    dy = np.zeros_like(plane)
    dx[:-1, :-1] = plane[:-1, :-1] - plane[:-1, 1:]
    dy[:-1, :-1] = plane[:-1, :-1] - plane[1:, :-1]
    tsv = (dx * dx + dy * dy).astype(np.float32)
    tsv[-1, :] = plane[-1, :]
    tsv[:, -1] = plane[:, -1]
    ent = (plane * np.log(plane / np.float32(0.001))).astype(np.float32)
    refs = {2: float(tsv[m].astype(np.float64).sum()), 1: float(ent[m].astype(np.float64).sum())}
    d_plane = torch.from_numpy(plane).cuda()
    d_noise = torch.from_numpy(noise).cuda()
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for call in range(2):
        for kind, G, eta in ((2, 0.0, 0.0), (1, 0.001, -1.0)):
            out.fill_(-1.0)
            rc = fn(kind, C.c_void_p(d_plane.data_ptr()), C.c_void_p(d_noise.data_ptr()), cut, n,
                    G, eta, 0.0, C.c_void_p(out.data_ptr()), stream)
            assert rc == 0, L.gv_last_error()
            torch.cuda.synchronize()
            got = float(out.item())
            assert abs(got - refs[kind]) <= 1e-5 * abs(refs[kind]), (call, kind, got, refs[kind])


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
