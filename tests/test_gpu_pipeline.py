"""The one-call entry points' copy/compute pipelines (pairwise: chunks of
pairs uploaded while earlier chunks compute; cdist: result rows copied back
while later query chunks compute), from pinned and from pageable host
buffers: identical to the resident-state runs and to the oracle."""
import ctypes

import numpy as np
import pytest

import oracle
from editdist_bench_gb300 import _lib, gpu, workloads as W

pytestmark = pytest.mark.gpu

CODE = {"int32": 0, "uint16": 1, "uint8": 2}


class _Pinned:
    def __init__(self):
        self.ctx = _lib.context()
        self.ptrs = []

    def empty(self, n, dtype):
        dtype = np.dtype(dtype)
        nbytes = max(1, n * dtype.itemsize)
        p = ctypes.c_void_p()
        self.ctx.check(self.ctx.lib.blg_host_alloc(self.ctx.h, ctypes.c_size_t(nbytes), ctypes.byref(p)))
        self.ptrs.append(p.value)
        raw = (ctypes.c_uint8 * nbytes).from_address(p.value)
        return np.frombuffer(raw, dtype=np.uint8)[:n * dtype.itemsize].view(dtype)

    def copy(self, a):
        out = self.empty(a.size, a.dtype)
        out[:] = a.ravel()
        return out

    def free(self):
        for p in self.ptrs:
            self.ctx.check(self.ctx.lib.blg_host_free(self.ctx.h, p))
        self.ptrs = []


@pytest.fixture
def pinned(gpu):
    p = _Pinned()
    yield p
    p.free()


def _pairwise_call(a, b, k, dt, out):
    ctx = _lib.context()
    (ba, oa), (bb, ob) = a, b
    ctx.check(ctx.lib.blg_pairwise(ctx.h, ba.ctypes.data, oa.ctypes.data, bb.ctypes.data, ob.ctypes.data,
                                   len(oa) - 1, -1 if k is None else k, CODE[dt], out.ctypes.data, None))
    return out


def _cdist_call(q, c, k, dt, out):
    ctx = _lib.context()
    (bq, oq), (bc, oc) = q, c
    ctx.check(ctx.lib.blg_cdist(ctx.h, bq.ctypes.data, oq.ctypes.data, len(oq) - 1, bc.ctypes.data,
                                oc.ctypes.data, len(oc) - 1, -1 if k is None else k, CODE[dt],
                                out.ctypes.data, None))
    return out


@pytest.mark.parametrize("k,dt", [(None, "int32"), (3, "uint8")])
def test_pairwise_pipeline_pinned_and_pageable(pinned, k, dt):
    w = W.config1(n=300001, seed=41)                      # above the pipeline threshold, odd count
    want = oracle.saturate(oracle.pairs(w.a, w.b, k, threads=8), dt)
    pa = (pinned.copy(w.a[0]), pinned.copy(w.a[1]))
    pb = (pinned.copy(w.b[0]), pinned.copy(w.b[1]))
    out = pinned.empty(w.n, dt)
    np.testing.assert_array_equal(_pairwise_call(pa, pb, k, dt, out), want)
    np.testing.assert_array_equal(_pairwise_call(w.a, w.b, k, dt, np.empty(w.n, dt)), want)


@pytest.mark.parametrize("k,dt", [(None, "uint8"), (2, "uint16")])
def test_cdist_pipeline_matches_resident(pinned, k, dt):
    w = W.config2(nq=1027, nc=65536, seed=43)              # >= 64 MiB of results, 8 uneven chunks
    s = gpu.SearchBatch(w.q, w.c)
    ref = s.run(s.alloc(dt), max_dist=k).get()
    q = (pinned.copy(w.q[0]), pinned.copy(w.q[1]))
    c = (pinned.copy(w.c[0]), pinned.copy(w.c[1]))
    out = pinned.empty(w.nq * w.nc, dt).reshape(w.nq, w.nc)
    np.testing.assert_array_equal(_cdist_call(q, c, k, dt, out), ref)
    rows = [0, 128, 129, 700, 1026]
    np.testing.assert_array_equal(ref[rows], oracle.saturate(oracle.cross(W.take(w.q, rows), w.c, k, threads=8), dt))


@pytest.mark.parametrize("sched", ["auto", "plain", "lensort"])
def test_pairwise_pipeline_every_schedule(pinned, sched):
    """Uneven lengths (the banded and lane-spread solvers, not the tile
    kernel) through the chunked one-call path under each schedule."""
    w = W.config3(n=(1 << 18) + 3, seed=47)
    want = oracle.saturate(oracle.pairs(w.a, w.b, 8, threads=8), "uint8")
    pa = (pinned.copy(w.a[0]), pinned.copy(w.a[1]))
    pb = (pinned.copy(w.b[0]), pinned.copy(w.b[1]))
    out = pinned.empty(w.n, "uint8")
    gpu.set_schedule(sched)
    try:
        np.testing.assert_array_equal(_pairwise_call(pa, pb, 8, "uint8", out), want)
        np.testing.assert_array_equal(_pairwise_call(pa, pb, None, "int32", pinned.empty(w.n, "int32")),
                                      oracle.pairs(w.a, w.b, None, threads=8))
    finally:
        gpu.set_schedule("auto")
