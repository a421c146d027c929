"""4-bit results (BLG_UINT4): two results per byte, saturating at 15, so for
max_dist <= 14 every value is exact and the copy back is half of uint8's.
Checked against the oracle and against the uint8 output of the same call:
small and pipelined one-call searches (including an odd choice count, where
query chunks must end on even rows), pairwise with an odd pair count, and
the resident runs."""
import ctypes

import numpy as np
import pytest

import oracle
from editdist_bench_gb300 import _lib, workloads as W

pytestmark = pytest.mark.gpu


def _sat15(x):
    return np.minimum(x, 15).astype(np.uint8)


@pytest.mark.parametrize("k", [None, 2, 14])
def test_cdist_u4_small(gpu, k):
    rng = np.random.default_rng(61)
    q = W.random_strings(rng, rng.integers(0, 150, 33))
    c = W.concat(W.mutate(rng, q, 0.05), W.random_strings(rng, rng.integers(0, 150, 501)))
    got = gpu.cdist_u4_packed(q, c, max_dist=k)
    assert got.dtype == np.uint8 and got.shape == ((33 * 534 + 1) // 2,)
    np.testing.assert_array_equal(gpu.unpack_u4(got, 33 * 534), _sat15(oracle.cross(q, c, k)).ravel())


def test_cdist_u4_pipelined_odd_choice_count(gpu):
    """1024 queries x 65537 choices (odd): 64 Mi results, so the one-call
    pipeline runs in query chunks whose boundaries must be even rows."""
    w = W.config4(nq=1024, nc=65537, seed=62)
    got = gpu.unpack_u4(gpu.cdist_u4_packed(w.q, w.c, max_dist=4), w.nq * w.nc).reshape(w.nq, w.nc)
    full8 = gpu.cdist_packed(w.q, w.c, max_dist=4, dtype="uint8")
    np.testing.assert_array_equal(got, _sat15(full8))
    rows = [0, 1, 511, 1022, 1023]
    np.testing.assert_array_equal(got[rows], _sat15(oracle.cross(W.take(w.q, rows), w.c, 4, threads=8)))


def test_pairwise_u4(gpu):
    rng = np.random.default_rng(63)
    for n in (1, 7, 4097, (1 << 18) + 1):
        a = W.random_strings(rng, rng.integers(0, 120, n))
        b = W.mutate(rng, a, rng.uniform(0, 0.2, n))
        got = gpu.pairwise_u4_packed(a, b, max_dist=9)
        assert got.shape == ((n + 1) // 2,)
        np.testing.assert_array_equal(gpu.unpack_u4(got, n), _sat15(oracle.pairs(a, b, 9)))


def test_resident_runs_u4(gpu):
    ctx = _lib.context()
    rng = np.random.default_rng(64)
    q = W.random_strings(rng, rng.integers(1, 100, 21))
    c = W.concat(W.mutate(rng, q, 0.1), W.random_strings(rng, rng.integers(1, 100, 300)))
    a = W.random_strings(rng, rng.integers(0, 90, 1001))
    b = W.mutate(rng, a, 0.1)

    def dev(nbytes):
        p = ctypes.c_void_p()
        ctx.check(ctx.lib.blg_malloc(ctx.h, nbytes, ctypes.byref(p)))
        return p.value

    s = gpu.SearchBatch(q, c)
    n = s.nq * s.nc
    d = dev((n + 1) // 2)
    for k in (3, None):
        ctx.check(ctx.lib.blg_search_run(ctx.h, s.h, -1 if k is None else k, _lib.UINT4, d))
        got = np.empty((n + 1) // 2, dtype=np.uint8)
        ctx.check(ctx.lib.blg_memcpy_d2h(ctx.h, got.ctypes.data, d, got.nbytes))
        np.testing.assert_array_equal(gpu.unpack_u4(got, n), _sat15(oracle.cross(q, c, k)).ravel())
    ctx.check(ctx.lib.blg_free(ctx.h, d))
    pb = gpu.PairsBatch(a, b)
    d = dev((1001 + 1) // 2)
    ctx.check(ctx.lib.blg_pairs_run(ctx.h, pb.h, 5, _lib.UINT4, d))
    got = np.empty(501, dtype=np.uint8)
    ctx.check(ctx.lib.blg_memcpy_d2h(ctx.h, got.ctypes.data, d, got.nbytes))
    ctx.check(ctx.lib.blg_free(ctx.h, d))
    np.testing.assert_array_equal(gpu.unpack_u4(got, 1001), _sat15(oracle.pairs(a, b, 5)))
