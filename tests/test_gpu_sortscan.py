"""The device sort, scan and run-length primitives of the set-up passes
(gridding, weighting, visibility ordering) against numpy: a stable sort on
the selected key bits (numpy's stable argsort), exclusive prefix sums and
runs of equal keys, over ragged sizes around the 4096-key chunks, skewed
and uniform keys, and key bits outside the sorted range."""

import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

SIZES = [1, 2, 31, 4095, 4096, 4097, 2048 * 3 + 5, 100_003, 1_234_567]


def _lib():
    import gpuvmem_gb300 as gv
    L = gv.lib()
    vp, i32, i64 = C.c_void_p, C.c_int32, C.c_int64
    for name, args in {
        "gv_radix_sort_pairs_u32": [vp, vp, vp, vp, i64, i32, i32, vp],
        "gv_radix_sort_pairs_u64": [vp, vp, vp, vp, i64, i32, i32, vp],
        "gv_exclusive_scan_i32": [vp, vp, i64, vp],
        "gv_run_length_encode_u32": [vp, i64, vp, vp, vp, i64, vp, vp],
    }.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = C.c_int
    return L


def _check(st):
    import gpuvmem_gb300 as gv
    gv.check(st)


def _dev(a):
    """numpy uint32 / uint64 / int64 / int32 array -> cuda tensor of the same bytes"""
    view = {np.dtype(np.uint32): np.int32, np.dtype(np.uint64): np.int64}.get(a.dtype, a.dtype)
    return torch.from_numpy(np.ascontiguousarray(a).view(view)).cuda()


def _host(t, dtype):
    return t.cpu().numpy().view(dtype)


def _sort32(keys, vals, b0, b1):
    L = _lib()
    n = keys.size
    ki, vi = _dev(keys), _dev(vals)
    ko, vo = torch.empty_like(ki), torch.empty_like(vi)
    _check(L.gv_radix_sort_pairs_u32(ki.data_ptr(), ko.data_ptr(), vi.data_ptr(), vo.data_ptr(),
                                     n, b0, b1, None))
    return _host(ko, np.uint32), _host(vo, np.uint32)


def _expect(keys, vals, b0, b1):
    sel = (keys.astype(np.uint64) >> np.uint64(b0))
    if b1 - b0 < 64:
        sel &= np.uint64((1 << (b1 - b0)) - 1)
    order = np.argsort(sel, kind="stable")
    return keys[order], vals[order]


def _keysets(n, rng):
    yield "uniform", rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
    yield "few", rng.integers(0, 7, n).astype(np.uint32)
    yield "equal", np.full(n, 0xDEADBEEF, np.uint32)
    yield "sorted", np.sort(rng.integers(0, 1 << 22, n)).astype(np.uint32)
    yield "reversed", np.sort(rng.integers(0, 1 << 22, n))[::-1].astype(np.uint32)
    # gridding-like: cells of a 2048^2 grid clustered near its centre, and
    # the all-ones key of taps outside the grid
    c = np.clip(rng.normal(2048 * 1024 + 1024, 20000.0, n), 0, 2048 * 2048 - 1).astype(np.uint32)
    c[rng.random(n) < 0.05] = 0xFFFFFFFF
    yield "cells", c


@pytest.mark.parametrize("n", SIZES)
def test_sort_u32_full_keys(n):
    rng = np.random.default_rng(n)
    for name, keys in _keysets(n, rng):
        vals = np.arange(n, dtype=np.uint32) ^ np.uint32(0x5A5A5A5A)
        k, v = _sort32(keys, vals, 0, 32)
        ek, ev = _expect(keys, vals, 0, 32)
        assert np.array_equal(k, ek), name
        assert np.array_equal(v, ev), name


@pytest.mark.parametrize("bits", [(0, 23), (0, 1), (3, 17), (8, 16), (0, 0)])
def test_sort_u32_bit_ranges(bits):
    """bits outside [begin, end) do not order; the keys move whole"""
    b0, b1 = bits
    rng = np.random.default_rng(7 + b0 + 32 * b1)
    for n in (4097, 300_001):
        keys = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
        vals = np.arange(n, dtype=np.uint32)
        k, v = _sort32(keys, vals, b0, b1)
        ek, ev = _expect(keys, vals, b0, b1)
        assert np.array_equal(k, ek)
        assert np.array_equal(v, ev)


def test_sort_u32_largest_gridding_slab():
    """2^27 pairs, the gridding's largest slab, on its 23 cell bits: checked
    by properties (sorted on the bits, equal keys in input order, a
    permutation carrying its keys) instead of a host sort of that size"""
    n = 1 << 27
    rng = np.random.default_rng(27)
    keys = rng.integers(0, 1 << 23, n, dtype=np.uint32)
    keys[rng.random(n) < 0.01] = 0xFFFFFFFF
    k, v = _sort32(keys, np.arange(n, dtype=np.uint32), 0, 23)
    sel = k & np.uint32((1 << 23) - 1)
    assert np.all(sel[1:] >= sel[:-1])
    same = sel[1:] == sel[:-1]
    assert np.all(v[1:][same] > v[:-1][same])
    assert np.all(np.bincount(v, minlength=n) == 1)
    assert np.array_equal(keys[v], k)


@pytest.mark.parametrize("n", [1, 2047, 2048, 2049, 500_003])
def test_sort_u64(n):
    L = _lib()
    rng = np.random.default_rng(100 + n)
    sets = [rng.integers(0, 2**64, n, dtype=np.uint64),
            (rng.integers(0, 50, n).astype(np.uint64) << np.uint64(40)) |
            rng.integers(0, 1000, n).astype(np.uint64)]
    for keys in sets:
        vals = rng.integers(-2**62, 2**62, n, dtype=np.int64)
        for b0, b1 in ((0, 64), (20, 47)):
            ki, vi = _dev(keys), _dev(vals)
            ko, vo = torch.empty_like(ki), torch.empty_like(vi)
            _check(L.gv_radix_sort_pairs_u64(ki.data_ptr(), ko.data_ptr(), vi.data_ptr(),
                                             vo.data_ptr(), n, b0, b1, None))
            ek, ev = _expect(keys, vals, b0, b1)
            assert np.array_equal(_host(ko, np.uint64), ek)
            assert np.array_equal(_host(vo, np.int64), ev)


def test_sort_empty_and_invalid():
    L = _lib()
    t = torch.zeros(8, dtype=torch.int32, device="cuda")
    _check(L.gv_radix_sort_pairs_u32(t.data_ptr(), t.data_ptr(), t.data_ptr(), t.data_ptr(),
                                     0, 0, 32, None))
    assert L.gv_radix_sort_pairs_u32(t.data_ptr(), t.data_ptr(), t.data_ptr(), t.data_ptr(),
                                     8, 0, 33, None) != 0
    assert L.gv_radix_sort_pairs_u32(None, None, None, None, 8, 0, 32, None) != 0


@pytest.mark.parametrize("n", [1, 2, 4095, 4096, 4097, 1_000_007, 4 * 2048 * 2048 + 3])
def test_exclusive_scan(n):
    L = _lib()
    rng = np.random.default_rng(n)
    a = rng.integers(0, 3, n).astype(np.int32)
    d = _dev(a)
    out = torch.empty_like(d)
    _check(L.gv_exclusive_scan_i32(d.data_ptr(), out.data_ptr(), n, None))
    e = np.concatenate([[0], np.cumsum(a[:-1], dtype=np.int64)]).astype(np.int32)
    assert np.array_equal(out.cpu().numpy(), e)
    # in place
    _check(L.gv_exclusive_scan_i32(d.data_ptr(), d.data_ptr(), n, None))
    assert np.array_equal(d.cpu().numpy(), e)


@pytest.mark.parametrize("n", [1, 5, 4097, 777_777])
def test_run_length_encode(n):
    L = _lib()
    rng = np.random.default_rng(3 * n)
    keys = np.sort(rng.integers(0, max(1, n // 5), n)).astype(np.uint32)
    keys[-min(n, 3):] = 0xFFFFFFFF
    starts = np.flatnonzero(np.concatenate([[True], keys[1:] != keys[:-1]]))
    lengths = np.diff(np.concatenate([starts, [n]]))
    for cap in (n, len(starts), max(1, len(starts) // 2)):
        d = _dev(keys)
        rk = torch.zeros(cap, dtype=torch.int32, device="cuda")
        rs, rl = torch.zeros_like(rk), torch.zeros_like(rk)
        nr = torch.zeros(1, dtype=torch.int32, device="cuda")
        _check(L.gv_run_length_encode_u32(d.data_ptr(), n, rk.data_ptr(), rs.data_ptr(),
                                          rl.data_ptr(), cap, nr.data_ptr(), None))
        assert int(nr.item()) == len(starts)
        m = min(cap, len(starts))
        assert np.array_equal(_host(rk, np.uint32)[:m], keys[starts][:m])
        assert np.array_equal(_host(rs, np.uint32)[:m], starts[:m])
        assert np.array_equal(_host(rl, np.uint32)[:m], lengths[:m])
