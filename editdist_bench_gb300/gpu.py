"""GB300 versions of ``pairwise`` and ``cdist`` — a drop-in for ``bitlev.gpu``.

    from editdist_bench_gb300 import gpu
    d = gpu.cdist(queries, choices, max_dist=2, dtype="uint8")

Same signatures and results as bitlev/gpu.py:36-138: ``max_dist=k`` returns
min(d, k+1); int32, uint16 or uint8 output with saturation;
``return_device=True`` keeps the result in GPU memory (a ``DeviceArray``
with ``__cuda_array_interface__``). Differences, all deliberate:

* the work runs in ``libbitlev_gb300.so`` (C-ABI, ctypes), not CuPy/NVRTC;
* every length runs on the GPU (the reference computes pairs whose shorter
  string exceeds 256, and queries longer than 512, on the CPU);
* uint16 saturation is fused into the kernels' stores.

The packed entry points (``pairwise_packed``/``cdist_packed``) and the
resident ``PairsBatch``/``SearchBatch`` mirror the reference benchmark's
``PairsState``/``CrossState`` (bench/cudamyers.py:83-174).
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

from . import _common, _lib
from ._common import DTYPE_CODE, as_list, check_dtype, check_k, pack
from .device_array import DeviceArray

__all__ = ["available", "pairwise", "cdist", "pairwise_packed", "cdist_packed", "PairsBatch",
           "SearchBatch", "ProblemBatch", "cdist_batch", "pack", "set_schedule", "synchronize"]


def available() -> bool:
    """True when the CUDA library is built and a GPU is visible."""
    return _lib.device_count() > 0


def _c(a: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(a)


def _packed(p):
    buf, off = p
    return _c(np.asarray(buf, dtype=np.uint8)), _c(np.asarray(off, dtype=np.int64))


def _empty(shape, dt, return_device, ctx=None):
    if return_device:
        return DeviceArray(0, shape, dt, ctx or _lib.context())
    return np.empty(shape, dtype=dt)


def pairwise_packed(pa, pb, max_dist=None, dtype=np.int32, return_device: bool = False):
    """out[i] = d(a_i, b_i) for packed inputs ``(buf uint8, off int64[n+1])``."""
    (ba, oa), (bb, ob) = _packed(pa), _packed(pb)
    n = len(oa) - 1
    if len(ob) - 1 != n:
        raise ValueError(f"length mismatch: {n} vs {len(ob) - 1}")
    k, dt = check_k(max_dist), check_dtype(dtype)
    ctx = _lib.context()
    if n == 0:
        return _empty((0,), dt, return_device, ctx)
    lib = ctx.lib
    if return_device:
        dptr = ctypes.c_void_p()
        ctx.check(lib.blg_pairwise(ctx.h, ba.ctypes.data, oa.ctypes.data, bb.ctypes.data,
                                   ob.ctypes.data, n, k, DTYPE_CODE[dt], None, ctypes.byref(dptr)),
                  "pairwise")
        return DeviceArray(dptr.value, (n,), dt, ctx)
    out = np.empty(n, dtype=dt)
    ctx.check(lib.blg_pairwise(ctx.h, ba.ctypes.data, oa.ctypes.data, bb.ctypes.data,
                               ob.ctypes.data, n, k, DTYPE_CODE[dt], out.ctypes.data, None),
              "pairwise")
    return out


def cdist_packed(pq, pc, max_dist=None, dtype=np.int32, return_device: bool = False):
    """out[i, j] = d(q_i, c_j) for packed inputs."""
    (bq, oq), (bc, oc) = _packed(pq), _packed(pc)
    nq, nc = len(oq) - 1, len(oc) - 1
    k, dt = check_k(max_dist), check_dtype(dtype)
    ctx = _lib.context()
    if nq == 0 or nc == 0:
        return _empty((nq, nc), dt, return_device, ctx)
    lib = ctx.lib
    if return_device:
        dptr = ctypes.c_void_p()
        ctx.check(lib.blg_cdist(ctx.h, bq.ctypes.data, oq.ctypes.data, nq, bc.ctypes.data,
                                oc.ctypes.data, nc, k, DTYPE_CODE[dt], None, ctypes.byref(dptr)),
                  "cdist")
        return DeviceArray(dptr.value, (nq, nc), dt, ctx)
    out = np.empty((nq, nc), dtype=dt)
    ctx.check(lib.blg_cdist(ctx.h, bq.ctypes.data, oq.ctypes.data, nq, bc.ctypes.data,
                            oc.ctypes.data, nc, k, DTYPE_CODE[dt], out.ctypes.data, None),
              "cdist")
    return out


# ---- 4-bit results (BLG_UINT4): two per byte, saturating at 15; exact for
#      max_dist <= 14. Half the bytes of uint8 cross from the device.
def unpack_u4(packed: np.ndarray, n: int) -> np.ndarray:
    """uint8[n] from 4-bit results packed two per byte (low nibble first)."""
    p = np.asarray(packed, dtype=np.uint8)
    out = np.empty(2 * len(p), dtype=np.uint8)
    out[0::2] = p & 15
    out[1::2] = p >> 4
    return out[:n]


def pairwise_u4_packed(pa, pb, max_dist=None) -> np.ndarray:
    """pairwise_packed with 4-bit results: uint8[(n + 1) // 2], two per byte."""
    (ba, oa), (bb, ob) = _packed(pa), _packed(pb)
    n = len(oa) - 1
    if len(ob) - 1 != n:
        raise ValueError(f"length mismatch: {n} vs {len(ob) - 1}")
    k = check_k(max_dist)
    ctx = _lib.context()
    out = np.zeros(max(1, (n + 1) // 2), dtype=np.uint8)
    if n:
        ctx.check(ctx.lib.blg_pairwise(ctx.h, ba.ctypes.data, oa.ctypes.data, bb.ctypes.data, ob.ctypes.data, n, k,
                                       _lib.UINT4, out.ctypes.data, None), "pairwise")
    return out[:(n + 1) // 2]


def cdist_u4_packed(pq, pc, max_dist=None) -> np.ndarray:
    """cdist_packed with 4-bit results: uint8[(nq * nc + 1) // 2], row-major,
    two results per byte."""
    (bq, oq), (bc, oc) = _packed(pq), _packed(pc)
    nq, nc = len(oq) - 1, len(oc) - 1
    k = check_k(max_dist)
    ctx = _lib.context()
    out = np.zeros(max(1, (nq * nc + 1) // 2), dtype=np.uint8)
    if nq and nc:
        ctx.check(ctx.lib.blg_cdist(ctx.h, bq.ctypes.data, oq.ctypes.data, nq, bc.ctypes.data, oc.ctypes.data, nc,
                                    k, _lib.UINT4, out.ctypes.data, None), "cdist")
    return out[:(nq * nc + 1) // 2]


# one record of blg_cdist_matches / blg_search_matches (include/bitlev_gb300.h: blg_match)
MATCH_DTYPE = np.dtype([("query", "<i8"), ("choice", "<i8"), ("dist", "<i4"), ("reserved", "<i4")])


def _match_k(max_dist) -> int:
    k = check_k(max_dist)
    if k < 0:
        raise ValueError("matches need a max_dist (>= 0); the exact result is the dense cdist")
    return k


def cdist_matches_packed(pq, pc, max_dist, capacity: int | None = None):
    """Every (query, choice) with d(q, c) <= max_dist, sorted by (query,
    choice): arrays (query, choice, dist). Packed inputs. The records are
    found on the GPU; only they cross to the host, not the nq x nc matrix."""
    (bq, oq), (bc, oc) = _packed(pq), _packed(pc)
    nq, nc = len(oq) - 1, len(oc) - 1
    k = _match_k(max_dist)
    ctx = _lib.context()
    cap = capacity if capacity is not None else min(max(nq, nc, 1) * 4, nq * nc, 1 << 20)
    while True:
        rec = np.empty(max(cap, 0), dtype=MATCH_DTYPE)
        cnt = ctypes.c_int64()
        ctx.check(ctx.lib.blg_cdist_matches(ctx.h, bq.ctypes.data, oq.ctypes.data, nq, bc.ctypes.data,
                                            oc.ctypes.data, nc, k, rec.ctypes.data if cap else None, cap,
                                            ctypes.byref(cnt)), "cdist_matches")
        if cnt.value <= cap or capacity is not None:
            rec = rec[:min(cnt.value, cap)]
            return rec["query"].copy(), rec["choice"].copy(), rec["dist"].copy()
        cap = cnt.value


def cdist_matches(queries, choices, max_dist, capacity: int | None = None):
    """(query, choice, dist) of every pair within max_dist — the matches-only
    form of cdist(queries, choices, max_dist)."""
    q, c = as_list(queries), as_list(choices)
    _match_k(max_dist)
    return cdist_matches_packed(pack(q), pack(c), max_dist, capacity)


# Page-locked staging of the list API's packed inputs: the native packer
# writes each string's bytes straight into it, so the one-call entry points
# copy them to the device at full link speed. Grown on demand and kept for
# the process (reused by every call; calls take turns on it).
_stage_lock = threading.Lock()
_stage = {}


def _pinned(ctx, slot: str, nbytes: int) -> int:
    ptr, cap = _stage.get(slot, (None, 0))
    if cap < nbytes:
        if ptr:
            ctx.lib.blg_host_free(ctx.h, ptr)
            _stage.pop(slot)
        cap = max(nbytes, 2 * cap, 1 << 16)
        p = ctypes.c_void_p()
        ctx.check(ctx.lib.blg_host_alloc(ctx.h, ctypes.c_size_t(cap), ctypes.byref(p)), "host_alloc")
        ptr = p.value
        _stage[slot] = (ptr, cap)
    return ptr


def _pack_pinned(ctx, seq, slot: str):
    """(buf address, offsets address, n) of `seq` packed into pinned staging."""
    n, total = _common._blgpack.size(seq)
    bp = _pinned(ctx, slot + "/buf", max(total, 1))
    op = _pinned(ctx, slot + "/off", 8 * (n + 1))
    _common._blgpack.pack_into(seq, bp, max(total, 1), op)
    return bp, op, n


def pairwise(a, b, max_dist=None, dtype=np.int32, return_device: bool = False):
    """out[i] = d(a[i], b[i]) on the GPU (bitlev/gpu.py:71-103)."""
    a, b = as_list(a), as_list(b)
    if len(a) != len(b):
        raise ValueError(f"length mismatch: {len(a)} vs {len(b)}")
    k, dt = check_k(max_dist), check_dtype(dtype)
    if len(a) == 0:
        return _empty((0,), dt, return_device)
    if _common._blgpack is None:
        return pairwise_packed(pack(a), pack(b), k if k >= 0 else None, dt, return_device)
    ctx = _lib.context()
    n = len(a)
    with _stage_lock:
        ba, oa, _ = _pack_pinned(ctx, a, "a")
        bb, ob, _ = _pack_pinned(ctx, b, "b")
        if return_device:
            dptr = ctypes.c_void_p()
            ctx.check(ctx.lib.blg_pairwise(ctx.h, ba, oa, bb, ob, n, k, DTYPE_CODE[dt], None, ctypes.byref(dptr)),
                      "pairwise")
            return DeviceArray(dptr.value, (n,), dt, ctx)
        out = np.empty(n, dtype=dt)
        ctx.check(ctx.lib.blg_pairwise(ctx.h, ba, oa, bb, ob, n, k, DTYPE_CODE[dt], out.ctypes.data, None),
                  "pairwise")
        return out


def cdist(queries, choices, max_dist=None, dtype=np.int32, return_device: bool = False):
    """out[i, j] = d(queries[i], choices[j]) on the GPU (bitlev/gpu.py:106-138)."""
    q, c = as_list(queries), as_list(choices)
    k, dt = check_k(max_dist), check_dtype(dtype)
    if not q or not c:
        return _empty((len(q), len(c)), dt, return_device)
    if _common._blgpack is None:
        return cdist_packed(pack(q), pack(c), k if k >= 0 else None, dt, return_device)
    ctx = _lib.context()
    nq, nc = len(q), len(c)
    with _stage_lock:
        bq, oq, _ = _pack_pinned(ctx, q, "q")
        bc, oc, _ = _pack_pinned(ctx, c, "c")
        if return_device:
            dptr = ctypes.c_void_p()
            ctx.check(ctx.lib.blg_cdist(ctx.h, bq, oq, nq, bc, oc, nc, k, DTYPE_CODE[dt], None, ctypes.byref(dptr)),
                      "cdist")
            return DeviceArray(dptr.value, (nq, nc), dt, ctx)
        out = np.empty((nq, nc), dtype=dt)
        ctx.check(ctx.lib.blg_cdist(ctx.h, bq, oq, nq, bc, oc, nc, k, DTYPE_CODE[dt], out.ctypes.data, None),
                  "cdist")
        return out


class PairsBatch:
    """Packed pairs resident in HBM (bench/cudamyers.py:83-114): upload once,
    ``run`` many times into a device buffer (stream-ordered, no sync)."""

    def __init__(self, pa, pb):
        (ba, oa), (bb, ob) = _packed(pa), _packed(pb)
        self.n = len(oa) - 1
        if len(ob) - 1 != self.n:
            raise ValueError(f"length mismatch: {self.n} vs {len(ob) - 1}")
        self.ctx = _lib.context()
        h = ctypes.c_void_p()
        self.ctx.check(self.ctx.lib.blg_pairs_upload(self.ctx.h, ba.ctypes.data, oa.ctypes.data,
                                                     bb.ctypes.data, ob.ctypes.data, self.n,
                                                     ctypes.byref(h)), "pairs_upload")
        self.h = h

    def alloc(self, dtype=np.int32) -> DeviceArray:
        dt = check_dtype(dtype)
        p = ctypes.c_void_p()
        self.ctx.check(self.ctx.lib.blg_malloc(self.ctx.h, max(1, self.n * dt.itemsize),
                                               ctypes.byref(p)), "malloc")
        return DeviceArray(p.value, (self.n,), dt, self.ctx)

    def run(self, out: DeviceArray, max_dist=None):
        k = check_k(max_dist)
        self.ctx.check(self.ctx.lib.blg_pairs_run(self.ctx.h, self.h, k, DTYPE_CODE[out.dtype],
                                                  out.ptr), "pairs_run")
        return out

    def __del__(self):
        if getattr(self, "h", None) and self.h.value:
            self.ctx.lib.blg_pairs_free(self.ctx.h, self.h)
            self.h = None


class SearchBatch:
    """Packed queries and choices resident in HBM (bench/cudamyers.py:139-174)."""

    def __init__(self, pq, pc):
        (bq, oq), (bc, oc) = _packed(pq), _packed(pc)
        self.nq, self.nc = len(oq) - 1, len(oc) - 1
        self.ctx = _lib.context()
        h = ctypes.c_void_p()
        self.ctx.check(self.ctx.lib.blg_search_upload(self.ctx.h, bq.ctypes.data, oq.ctypes.data,
                                                      self.nq, bc.ctypes.data, oc.ctypes.data,
                                                      self.nc, ctypes.byref(h)), "search_upload")
        self.h = h

    def alloc(self, dtype=np.int32) -> DeviceArray:
        dt = check_dtype(dtype)
        p = ctypes.c_void_p()
        self.ctx.check(self.ctx.lib.blg_malloc(self.ctx.h, max(1, self.nq * self.nc * dt.itemsize),
                                               ctypes.byref(p)), "malloc")
        return DeviceArray(p.value, (self.nq, self.nc), dt, self.ctx)

    def run(self, out: DeviceArray, max_dist=None):
        k = check_k(max_dist)
        self.ctx.check(self.ctx.lib.blg_search_run(self.ctx.h, self.h, k, DTYPE_CODE[out.dtype],
                                                   out.ptr), "search_run")
        return out

    def match_buffer(self, capacity: int) -> DeviceArray:
        """Device room for `capacity` match records."""
        p = ctypes.c_void_p()
        self.ctx.check(self.ctx.lib.blg_malloc(self.ctx.h, max(1, capacity * MATCH_DTYPE.itemsize),
                                               ctypes.byref(p)), "malloc")
        return DeviceArray(p.value, (capacity,), MATCH_DTYPE, self.ctx)

    def matches_into(self, buf: DeviceArray, max_dist) -> int:
        """Match records (d <= max_dist, sorted by (query, choice)) into the
        device buffer; returns the total number of matches (records past the
        buffer's length are not written)."""
        cnt = ctypes.c_int64()
        self.ctx.check(self.ctx.lib.blg_search_matches(self.ctx.h, self.h, _match_k(max_dist), buf.ptr,
                                                       buf.shape[0], ctypes.byref(cnt)), "search_matches")
        return cnt.value

    def matches(self, max_dist):
        """(query, choice, dist) arrays of every pair within max_dist."""
        buf = self.match_buffer(1 << 16)
        n = self.matches_into(buf, max_dist)
        if n > buf.shape[0]:
            buf = self.match_buffer(n)
            n = self.matches_into(buf, max_dist)
        rec = buf.get()[:n]
        return rec["query"].copy(), rec["choice"].copy(), rec["dist"].copy()

    def __del__(self):
        if getattr(self, "h", None) and self.h.value:
            self.ctx.lib.blg_search_free(self.ctx.h, self.h)
            self.h = None


class ProblemBatch:
    """Many independent cdist problems ``(queries, choices, max_dist, dtype)``
    (packed inputs) resident in HBM, with device outputs (``outputs``, one
    DeviceArray each). ``run()`` launches the whole batch as one CUDA graph
    around a persistent kernel (stream-ordered, no sync)."""

    def __init__(self, problems):
        self.ctx = _lib.context()
        self.outputs = []
        structs = []
        keep = []
        for pq, pc, max_dist, dtype in problems:
            (bq, oq), (bc, oc) = _packed(pq), _packed(pc)
            k, dt = check_k(max_dist), check_dtype(dtype)
            nq, nc = len(oq) - 1, len(oc) - 1
            p = ctypes.c_void_p()
            self.ctx.check(self.ctx.lib.blg_malloc(self.ctx.h, max(16, nq * nc * dt.itemsize), ctypes.byref(p)),
                           "malloc")
            out = DeviceArray(p.value, (nq, nc), dt, self.ctx)
            self.outputs.append(out)
            keep += [bq, oq, bc, oc]
            structs.append(_lib.Problem(bq.ctypes.data, oq.ctypes.data, nq, bc.ctypes.data, oc.ctypes.data, nc,
                                        k, DTYPE_CODE[dt], out.ptr))
        arr = (_lib.Problem * max(1, len(structs)))(*structs)
        h = ctypes.c_void_p()
        self.ctx.check(self.ctx.lib.blg_batch_upload(self.ctx.h, arr, len(structs), ctypes.byref(h)), "batch_upload")
        self.h = h
        self.pairs = int(self.ctx.lib.blg_batch_pairs(h))

    def run(self):
        self.ctx.check(self.ctx.lib.blg_batch_run(self.ctx.h, self.h), "batch_run")
        return self.outputs

    def __del__(self):
        if getattr(self, "h", None) and self.h.value:
            self.ctx.lib.blg_batch_free(self.ctx.h, self.h)
            self.h = None


def cdist_batch(problems, return_device: bool = True):
    """[cdist(q, c, k, dtype) for each problem] in one batched launch."""
    b = ProblemBatch(problems)
    b.run()
    synchronize()
    return b.outputs if return_device else [o.get() for o in b.outputs]


_SCHEDULES = {"auto": _lib.SCHED_AUTO, "plain": _lib.SCHED_PLAIN, "learned": _lib.SCHED_LEARNED,
              "lensort": _lib.SCHED_LENSORT}


def autotune(cache_path=None) -> dict:
    """Time candidate launch shapes on this GPU and keep the fastest for the
    process's context (see blg_autotune); with ``cache_path`` a cache for the
    same device and library version is reused, a fresh result written."""
    ctx = _lib.context()
    ctx.check(ctx.lib.blg_autotune(ctx.h, None if cache_path is None else os.fsencode(cache_path)), "autotune")
    return tuning()


def tuning() -> dict:
    """The context's current launch shapes."""
    ctx = _lib.context()
    v = (ctypes.c_int32 * 17)()
    ctx.check(ctx.lib.blg_get_tuning(ctx.h, v, 17), "get_tuning")
    return {"search_queries_per_cta": {w + 1: int(v[w]) for w in range(8)}, "survivor_ctas_per_sm": int(v[8]),
            "survivors_per_job": int(v[9]), "survivor_round_columns": int(v[13]), "band_ctas_per_sm": int(v[10]),
            "tile_shape": int(v[12]),
            # the max_dist axis: the shapes above serve max_dist <= 8 (survivor
            # search) and <= 15 (banded pairs); these the rest up to 31
            "survivor_ctas_per_sm_k9_31": int(v[14]), "survivor_round_columns_k9_31": int(v[15]),
            "band_ctas_per_sm_k16_31": int(v[16]),
            "source": {0: "defaults", 1: "timed", 2: "cache"}[int(v[11])]}


def set_schedule(name: str):
    """Work order of max_dist runs: "auto" (survivor compaction), "plain" (one
    thread per pair in natural order, the reference's schedule), "learned"
    (compaction + the scheduler network's predicted exit order) or
    "lensort" (compaction + length-difference order). Results never change."""
    ctx = _lib.context()
    ctx.check(ctx.lib.blg_set_schedule(ctx.h, _SCHEDULES[name]), "set_schedule")


def synchronize():
    ctx = _lib.context()
    ctx.check(ctx.lib.blg_synchronize(ctx.h), "synchronize")
