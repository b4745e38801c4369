"""hg_dem_candidate_pairs_static: the broadphase for callers that cannot
allocate device memory on the calling path (a fixed device-memory budget set
at start-up, or a timing-critical loop where cudaMalloc's device
synchronisation is not acceptable).

It keeps every temporary in one fixed array inside the library, so the test
checks that two calls in a row, with different inputs, return exactly what
the allocating entry point hg_dem_candidate_pairs returns (the candidate
pairs are integer lists, so the tolerance is exact equality), and that inputs
beyond the array's limit are rejected. This file is collected last so that a
failure here leaves every other test already run; it passes alone too.
"""
import ctypes

import numpy as np
import pytest

import libhybridgrains_gb300 as hg
from libhybridgrains_gb300 import _capi

pytestmark = pytest.mark.gpu


def boxes(seed, n, extent):
    rng = np.random.default_rng(seed)
    c = rng.uniform(0.0, extent, size=(n, 2))
    r = rng.uniform(0.9e-3, 1.1e-3, size=n)
    return np.ascontiguousarray(c - r[:, None]), np.ascontiguousarray(c + r[:, None])


def static_pairs(ctx, mn, mx):
    lib = _capi.load()
    n = mn.shape[0]
    cnt = ctypes.c_int64()
    cap = 32 * n
    out = np.zeros((cap, 2), dtype=np.int32)
    st = lib.hg_dem_candidate_pairs_static(ctx._h, n, mn.ctypes.data_as(_capi._D),
                                           mx.ctypes.data_as(_capi._D), cap,
                                           out.ctypes.data_as(_capi._I32), ctypes.byref(cnt))
    assert st == 0, lib.hg_last_error()
    return out[: cnt.value]


def test_static_pairs_match_allocating_entry_point_twice(ctx):
    # two calls in a row: the second, smaller one must not see the first
    # call's leftovers in the shared array
    for seed, n, extent in ((1, 12000, 0.12), (2, 3000, 0.05)):
        mn, mx = boxes(seed, n, extent)
        ref = hg.candidate_pairs(ctx, mn, mx)
        got = static_pairs(ctx, mn, mx)
        assert len(ref) > 0
        assert np.array_equal(got, ref)


def test_static_pairs_rejects_too_many_boxes(ctx):
    lib = _capi.load()
    n = _capi.HG_STATIC_PAIRS_MAX_BOXES + 1
    mn, mx = boxes(3, n, 1.0)
    cnt = ctypes.c_int64()
    st = lib.hg_dem_candidate_pairs_static(ctx._h, n, mn.ctypes.data_as(_capi._D),
                                           mx.ctypes.data_as(_capi._D), 0, None,
                                           ctypes.byref(cnt))
    assert st == 4  # HG_ERR_CAPACITY
    assert b"at most" in lib.hg_last_error()


def call_static(ctx, mn, mx, cap):
    lib = _capi.load()
    n = mn.shape[0]
    cnt = ctypes.c_int64()
    out = np.zeros((max(cap, 1), 2), dtype=np.int32)
    st = lib.hg_dem_candidate_pairs_static(ctx._h, n, mn.ctypes.data_as(_capi._D),
                                           mx.ctypes.data_as(_capi._D), cap,
                                           out.ctypes.data_as(_capi._I32), ctypes.byref(cnt))
    return st, cnt.value, out[:cap]


def test_static_pairs_rejects_too_many_pairs(ctx):
    # 128 x 128 boxes of width 3.2 on a unit lattice: each overlaps its 48
    # neighbours within three cells, 24 of them later in index order (within
    # the per-box limit of 32), about 376,000 pairs in all
    k = np.arange(128, dtype=np.float64)
    c = np.stack(np.meshgrid(k, k), axis=-1).reshape(-1, 2)
    mn, mx = np.ascontiguousarray(c - 1.6), np.ascontiguousarray(c + 1.6)
    assert len(mn) <= _capi.HG_STATIC_PAIRS_MAX_BOXES
    ref = hg.candidate_pairs(ctx, mn, mx)
    assert len(ref) > _capi.HG_STATIC_PAIRS_MAX_PAIRS
    st, _, _ = call_static(ctx, mn, mx, 0)
    assert st == 4  # HG_ERR_CAPACITY
    assert b"holds at most" in _capi.load().hg_last_error()


def test_static_pairs_truncates_to_cap(ctx):
    # a cap below the count: the full count comes back, and the first cap
    # pairs of the sorted set
    mn, mx = boxes(1, 12000, 0.12)
    ref = hg.candidate_pairs(ctx, mn, mx)
    cap = 100
    assert len(ref) > cap
    st, count, got = call_static(ctx, mn, mx, cap)
    assert st == 0
    assert count == len(ref)
    assert np.array_equal(got, ref[:cap])
