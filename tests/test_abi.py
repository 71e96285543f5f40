"""The C-ABI library loads and exports every symbol include/*.h declares
(no compute calls: this runs without a GPU)."""

import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            txt = open(os.path.join(inc, f)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"\b(gv_[a-z0-9_]+)\s*\(", txt))
    return sorted(names)


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ["gv_problem_create", "gv_chi2", "gv_dchi2", "gv_objective", "gv_gradient",
              "gv_optimize", "gv_last_error"]:
        assert s in syms


def test_library_exports_every_declared_symbol():
    import gpuvmem_gb300 as gv
    if not os.path.exists(gv.LIB_PATH):
        pytest.fail("libgpuvmem_gb300.so is not built (run __graft_entry__.build())")
    L = ctypes.CDLL(gv.LIB_PATH)
    missing = [s for s in declared_symbols() if not hasattr(L, s)]
    assert not missing, missing
    assert set(gv.EXPORTS) <= set(declared_symbols())


def test_version_and_error_without_gpu():
    import gpuvmem_gb300 as gv
    L = gv.lib()
    assert b"sm_103a" in L.gv_version()
    # invalid arguments are rejected with a status, never an exit
    h = ctypes.c_void_p()
    assert L.gv_problem_create(None, ctypes.byref(h)) == 1
    assert b"null" in L.gv_last_error()
    assert L.gv_problem_destroy(None) == 0


def test_null_handles_are_rejected_without_gpu():
    """Every problem entry point validates its handle before touching the
    GPU: a null handle is GV_ERR_INVALID with a message, never a crash."""
    import gpuvmem_gb300 as gv
    L = gv.lib()
    f = ctypes.c_double()
    calls = [
        lambda: L.gv_objective(None, None, 0, ctypes.byref(f), None),
        lambda: L.gv_objective_many(None, None, 0, 0, ctypes.byref(f), None),
        lambda: L.gv_gradient(None, None, None, 0, 0),
        lambda: L.gv_evaluate(None, None, None, 0, 0, ctypes.byref(f), None),
        lambda: L.gv_dchi2(None, None, 0, None),
        lambda: L.gv_problem_set_graphs(None, 1),
        lambda: L.gv_linmin(None, None, None, 0, 1, ctypes.byref(ctypes.c_float()), None),
    ]
    for call in calls:
        assert call() == 1
        assert b"null" in L.gv_last_error()


def test_sort_scan_arguments_are_checked_without_gpu():
    """The device sort / scan / run-length entry points reject null buffers
    and negative sizes before any CUDA call, and an empty sort or scan is a
    no-op."""
    import gpuvmem_gb300 as gv
    L = gv.lib()
    vp, i32, i64 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64
    sigs = {"gv_radix_sort_pairs_u32": [vp, vp, vp, vp, i64, i32, i32, vp],
            "gv_radix_sort_pairs_u64": [vp, vp, vp, vp, i64, i32, i32, vp],
            "gv_exclusive_scan_i32": [vp, vp, i64, vp],
            "gv_run_length_encode_u32": [vp, i64, vp, vp, vp, i64, vp, vp]}
    for name, args in sigs.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = ctypes.c_int
    for fn in (L.gv_radix_sort_pairs_u32, L.gv_radix_sort_pairs_u64):
        assert fn(None, None, None, None, 0, 0, 32, None) == 0
        assert fn(None, None, None, None, 16, 0, 32, None) == 1
        assert b"null" in L.gv_last_error()
        assert fn(None, None, None, None, -1, 0, 32, None) == 1
    assert L.gv_exclusive_scan_i32(None, None, 0, None) == 0
    assert L.gv_exclusive_scan_i32(None, None, 5, None) == 1
    assert b"null" in L.gv_last_error()
    assert L.gv_run_length_encode_u32(None, 5, None, None, None, 5, None, None) == 1
    assert L.gv_run_length_encode_u32(None, -1, None, None, None, 5, None, None) == 1
