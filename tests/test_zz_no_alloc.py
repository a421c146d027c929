"""blg_cdist_noalloc: the cdist entry point for callers that cannot allocate
device memory (an engine that owns the GPU's memory and forbids its plugins
to call cudaMalloc, or a request path that must not block on or fail in an
allocation). The test owns the device buffers, as such a caller would, and
checks the results against the allocating entry point (blg_cdist) bit for
bit on two calls in a row — the second call reuses the fixed scratch that
the first one left behind. Kept in its own file, collected last."""
import ctypes

import numpy as np
import pytest

import oracle
from editdist_bench_gb300 import _lib, workloads as W

pytestmark = pytest.mark.gpu

_DT = {"int32": 0, "uint16": 1, "uint8": 2}


class DevBuf:
    """A device buffer the caller owns (allocated through the library's helper)."""

    def __init__(self, ctx, host: np.ndarray, extra: int = 0):
        self.ctx = ctx
        self.nbytes = host.nbytes + extra
        p = ctypes.c_void_p()
        ctx.check(ctx.lib.blg_malloc(ctx.h, max(16, self.nbytes), ctypes.byref(p)))
        self.ptr = p.value
        ctx.check(ctx.lib.blg_memset(ctx.h, self.ptr, 0, max(16, self.nbytes)))
        if host.nbytes:
            ctx.check(ctx.lib.blg_memcpy_h2d(ctx.h, self.ptr, host.ctypes.data, host.nbytes))

    def free(self):
        self.ctx.check(self.ctx.lib.blg_free(self.ctx.h, self.ptr))


def _noalloc(ctx, pq, pc, k, dt, off_shift=0, out_shift=0):
    """One blg_cdist_noalloc call on caller-owned device buffers. off_shift /
    out_shift place the query offsets / the output that many bytes past an
    aligned allocation (the checks of the entry point's alignment rules)."""
    (bq, oq), (bc, oc) = pq, pc
    nq, nc = len(oq) - 1, len(oc) - 1
    item = np.dtype(dt).itemsize
    bufs = [DevBuf(ctx, np.ascontiguousarray(bq[:oq[-1]]), 16), DevBuf(ctx, oq, 8),
            DevBuf(ctx, np.ascontiguousarray(bc[:oc[-1]]), 16), DevBuf(ctx, oc),
            DevBuf(ctx, np.zeros(nq * nc, dtype=dt), 16)]
    q, qo, c, co, out = bufs
    rc = ctx.lib.blg_cdist_noalloc(ctx.h, q.ptr, q.nbytes, qo.ptr + off_shift, nq, c.ptr, c.nbytes, co.ptr, nc,
                                   -1 if k is None else k, _DT[dt], out.ptr + out_shift)
    msg = ctx.lib.blg_last_error(ctx.h)          # read before the next call clears it
    got = np.empty((nq, nc), dtype=dt)
    if rc == 0:
        assert out_shift % item == 0
        ctx.check(ctx.lib.blg_memcpy_d2h(ctx.h, got.ctypes.data, out.ptr + out_shift, got.nbytes))
    for b in bufs:
        b.free()
    return rc, got, msg


def _alloc_entry(ctx, pq, pc, k, dt):
    (bq, oq), (bc, oc) = pq, pc
    nq, nc = len(oq) - 1, len(oc) - 1
    out = np.empty((nq, nc), dtype=dt)
    ctx.check(ctx.lib.blg_cdist(ctx.h, bq.ctypes.data, oq.ctypes.data, nq, bc.ctypes.data,
                                oc.ctypes.data, nc, -1 if k is None else k, _DT[dt],
                                out.ctypes.data, None))
    return out


def test_noalloc_matches_allocating_entry_point_twice(gpu):
    ctx = _lib.context()
    rng = np.random.default_rng(2026)
    # call 1: 300 queries (more than one 256-query chunk): the word and
    # limit boundaries of the query length (0, 1, 63..65, 128/129, 192/193,
    # 255, 256 — they pick the table width and the last-word variant), then
    # random lengths up to the 256-byte limit
    edges = [0, 1, 63, 64, 65, 128, 129, 192, 193, 255, 256]
    q1 = W.random_strings(rng, np.concatenate([edges, rng.integers(0, 257, 300 - len(edges))]))
    c1 = W.concat(W.mutate(rng, W.take(q1, rng.integers(0, 300, 200)), 0.05),
                  W.random_strings(rng, rng.integers(0, 300, 900)))
    # call 2: fewer, shorter queries, thresholded, narrow output
    q2 = W.random_strings(rng, rng.integers(0, 70, 37))
    c2 = W.concat(W.mutate(rng, q2, 0.1), W.random_strings(rng, rng.integers(0, 90, 500)))
    for pq, pc, k, dt in ((q1, c1, None, "int32"), (q2, c2, 3, "uint8")):
        rc, got, msg = _noalloc(ctx, pq, pc, k, dt)
        assert rc == 0, msg
        want = _alloc_entry(ctx, pq, pc, k, dt)
        np.testing.assert_array_equal(got, want)
    # and both against the oracle on the second call
    np.testing.assert_array_equal(got, oracle.saturate(oracle.cross(q2, c2, 3), "uint8"))


def test_noalloc_rejects_queries_beyond_its_scratch(gpu):
    ctx = _lib.context()
    rng = np.random.default_rng(5)
    q = W.random_strings(rng, [10, 257, 40])
    c = W.random_strings(rng, rng.integers(0, 80, 64))
    rc, _, msg = _noalloc(ctx, q, c, None, "int32")
    assert rc == _lib.ERR_ARG
    assert b"256 bytes" in msg
    # the context and the scratch stay usable
    rc, got, msg = _noalloc(ctx, W.take(q, [0, 2]), c, 2, "uint16")
    assert rc == 0, msg
    np.testing.assert_array_equal(got, _alloc_entry(ctx, W.take(q, [0, 2]), c, 2, "uint16"))


def test_noalloc_checks_alignment_before_running(gpu):
    """Offsets are read as int64: a pointer off an 8-byte boundary is refused
    before anything runs. A narrow output may start anywhere its element
    size allows (a row slice of a larger matrix): the stores fall back to
    single elements there."""
    ctx = _lib.context()
    rng = np.random.default_rng(9)
    q = W.random_strings(rng, rng.integers(0, 80, 9))
    c = W.concat(W.mutate(rng, q, 0.1), W.random_strings(rng, rng.integers(0, 80, 70)))
    rc, _, msg = _noalloc(ctx, q, c, None, "int32", off_shift=4)
    assert rc == _lib.ERR_ARG
    assert b"8-byte aligned" in msg
    rc, got, msg = _noalloc(ctx, q, c, 2, "uint8", out_shift=1)
    assert rc == 0, msg
    np.testing.assert_array_equal(got, _alloc_entry(ctx, q, c, 2, "uint8"))
    rc, got, msg = _noalloc(ctx, q, c, None, "uint16", out_shift=6)
    assert rc == 0, msg
    np.testing.assert_array_equal(got, _alloc_entry(ctx, q, c, None, "uint16"))
