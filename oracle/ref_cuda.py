"""The reference's OWN CUDA kernels, timed on this GPU — measurement
infrastructure, never the product.

bitlev launches its kernels through CuPy (bitlev/gpu.py:44-138), which is not
installable offline. This module loads the same kernels, compiled by
``oracle/build_oracle.py: build_ref_cuda()`` from csrc/gpu_kernels.cu where it
lies (a sm_103a cubin in ``oracle/_ref/``), through the CUDA driver API with
ctypes, and launches them with bitlev's geometry:

* pairwise (bitlev/gpu.py:71-103): pairs split by the shorter length into the
  classes <=16/32/64/128/256 (PAIR_CAPS, bitlev/gpu.py:22), an int32 index
  list per class, ``ed_pairs_c{CAP}`` with 256 threads and ceil(count/256)
  blocks, trimming on; pairs above 256 go to bitlev's CPU path there and are
  rejected here;
* cdist (bitlev/gpu.py:106-138): queries split by ceil(m/64) into the classes
  1/2/4/8 words (CROSS_NWS, :23), ``ed_cross_w{NW}`` with grid
  (queries in class, clamp(ceil(nc/256), 1, 64)), 256 threads and
  256*NW*8 bytes of dynamic shared memory; queries above 512 are rejected.

Outputs are int32, or uint8 (``out8``) as the kernels write them; bitlev makes
uint16 from int32 with a CuPy pass, which has no counterpart here (uint16
problems are timed as int32).  Timing: CUDA events around the launches of one
call with the inputs resident, L2 flushed between calls, like bench.py.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
CUBIN = os.path.join(HERE, "_ref", "ref_gpu_kernels.cubin")
PAIR_CAPS = (16, 32, 64, 128, 256)
CROSS_NWS = (1, 2, 4, 8)
THREADS = 256

_P = ctypes.c_void_p
_U64 = ctypes.c_uint64


def available() -> bool:
    return os.path.exists(CUBIN)


class _Driver:
    def __init__(self, device: int = 0):
        self.cu = ctypes.CDLL("libcuda.so.1")
        self._check(self.cu.cuInit(0), "cuInit")
        dev = ctypes.c_int()
        self._check(self.cu.cuDeviceGet(ctypes.byref(dev), device), "cuDeviceGet")
        self.ctx = _P()
        self._check(self.cu.cuDevicePrimaryCtxRetain(ctypes.byref(self.ctx), dev), "cuDevicePrimaryCtxRetain")
        self.dev = dev
        self._check(self.cu.cuCtxPushCurrent_v2(self.ctx), "cuCtxPushCurrent")
        self.mod = _P()
        self._check(self.cu.cuModuleLoad(ctypes.byref(self.mod), CUBIN.encode()), "cuModuleLoad")
        self.fn = {}
        self.cu.cuLaunchKernel.argtypes = [_P, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint, ctypes.c_uint,
                                           ctypes.c_uint, ctypes.c_uint, ctypes.c_uint, _P,
                                           ctypes.POINTER(_P), ctypes.POINTER(_P)]
        self.cu.cuMemcpyHtoD_v2.argtypes = [_U64, _P, ctypes.c_size_t]
        self.cu.cuMemcpyDtoH_v2.argtypes = [_P, _U64, ctypes.c_size_t]
        self.cu.cuMemFree_v2.argtypes = [_U64]
        self.cu.cuMemsetD8_v2.argtypes = [_U64, ctypes.c_ubyte, ctypes.c_size_t]

    @staticmethod
    def _check(rc, what):
        if rc != 0:
            raise RuntimeError(f"{what} failed: CUDA driver error {rc}")

    def function(self, name: str):
        if name not in self.fn:
            f = _P()
            self._check(self.cu.cuModuleGetFunction(ctypes.byref(f), self.mod, name.encode()), name)
            self.fn[name] = f
        return self.fn[name]

    def alloc(self, nbytes: int) -> int:
        p = _U64()
        self._check(self.cu.cuMemAlloc_v2(ctypes.byref(p), ctypes.c_size_t(max(1, nbytes))), "cuMemAlloc")
        return p.value

    def free(self, p: int):
        self.cu.cuMemFree_v2(p)

    def upload(self, a: np.ndarray) -> int:
        a = np.ascontiguousarray(a)
        p = self.alloc(a.nbytes)
        if a.nbytes:
            self._check(self.cu.cuMemcpyHtoD_v2(p, a.ctypes.data, a.nbytes), "cuMemcpyHtoD")
        return p

    def download(self, p: int, a: np.ndarray) -> np.ndarray:
        if a.nbytes:
            self._check(self.cu.cuMemcpyDtoH_v2(a.ctypes.data, p, a.nbytes), "cuMemcpyDtoH")
        return a

    def launch(self, name, grid, block, smem, args):
        vals = [ctypes.c_uint64(v) if kind == "p" else ctypes.c_int32(v) for kind, v in args]
        arr = (_P * len(vals))(*[ctypes.cast(ctypes.byref(v), _P) for v in vals])
        self._check(self.cu.cuLaunchKernel(self.function(name), grid[0], grid[1], 1, block, 1, 1, smem, None,
                                           arr, None), name)

    def close(self):
        if self.mod:
            self.cu.cuModuleUnload(self.mod)
            self.mod = None
            self.cu.cuCtxPopCurrent_v2(ctypes.byref(_P()))
            self.cu.cuDevicePrimaryCtxRelease_v2(self.dev)

    def sync(self):
        self._check(self.cu.cuCtxSynchronize(), "cuCtxSynchronize")

    def event(self):
        e = _P()
        self._check(self.cu.cuEventCreate(ctypes.byref(e), 0), "cuEventCreate")
        return e

    def elapsed_ms(self, a, b) -> float:
        ms = ctypes.c_float()
        self._check(self.cu.cuEventSynchronize(b), "cuEventSynchronize")
        self._check(self.cu.cuEventElapsedTime(ctypes.byref(ms), a, b), "cuEventElapsedTime")
        return ms.value


class RefCuda:
    """The reference's kernels on device `device`, launched as bitlev does."""

    def __init__(self, device: int = 0):
        if not available():
            raise FileNotFoundError(f"reference CUDA cubin not built: {CUBIN}")
        self.d = _Driver(device)
        self._flush = None
        self._bufs = []

    def _keep(self, p):
        self._bufs.append(p)
        return p

    def close(self):
        for p in self._bufs:
            self.d.free(p)
        self._bufs = []
        if self._flush:
            self.d.free(self._flush)
            self._flush = None
        self.d.close()

    # ---- pairwise
    def pairs_setup(self, a, b):
        (ba, oa), (bb, ob) = a, b
        n = len(oa) - 1
        m = np.minimum(np.diff(oa), np.diff(ob))
        cls = np.searchsorted(np.array(PAIR_CAPS), m)
        if n and cls.max() >= len(PAIR_CAPS):
            raise ValueError("pairs longer than 256 run on bitlev's CPU path, not timed here")
        st = {"n": n, "a": (self._keep(self.d.upload(ba)), self._keep(self.d.upload(oa))),
              "b": (self._keep(self.d.upload(bb)), self._keep(self.d.upload(ob))), "classes": []}
        for ci, cap in enumerate(PAIR_CAPS):
            idx = np.nonzero(cls == ci)[0].astype(np.int32)
            if len(idx):
                st["classes"].append((cap, len(idx), self._keep(self.d.upload(idx))))
        return st

    def pairs_run(self, st, out: int, k: int, out8: bool):
        for cap, cnt, idx in st["classes"]:
            self.d.launch(f"ed_pairs_c{cap}", ((cnt + THREADS - 1) // THREADS, 1), THREADS, 0,
                          [("p", st["a"][0]), ("p", st["a"][1]), ("p", st["b"][0]), ("p", st["b"][1]),
                           ("p", idx), ("i", cnt), ("p", out), ("i", 1), ("i", k), ("i", int(out8))])

    # ---- cdist
    def cross_setup(self, q, c):
        (bq, oq), (bc, oc) = q, c
        nq, nc = len(oq) - 1, len(oc) - 1
        words = (np.diff(oq) + 63) // 64
        cls = np.searchsorted(np.array(CROSS_NWS), words)
        if nq and cls.max() >= len(CROSS_NWS):
            raise ValueError("queries longer than 512 run on bitlev's CPU path, not timed here")
        st = {"nq": nq, "nc": nc, "q": (self._keep(self.d.upload(bq)), self._keep(self.d.upload(oq))),
              "c": (self._keep(self.d.upload(bc)), self._keep(self.d.upload(oc))), "classes": []}
        for ci, nw in enumerate(CROSS_NWS):
            idx = np.nonzero(cls == ci)[0].astype(np.int32)
            if len(idx):
                st["classes"].append((nw, len(idx), self._keep(self.d.upload(idx))))
        return st

    def cross_run(self, st, out: int, k: int, out8: bool):
        nc = st["nc"]
        gy = max(1, min((nc + THREADS - 1) // THREADS, 64))
        for nw, cnt, idx in st["classes"]:
            self.d.launch(f"ed_cross_w{nw}", (cnt, gy), THREADS, 256 * nw * 8,
                          [("p", st["q"][0]), ("p", st["q"][1]), ("p", idx), ("p", st["c"][0]), ("p", st["c"][1]),
                           ("i", nc), ("p", out), ("i", k), ("i", int(out8))])

    # ---- timing
    def time_calls(self, run, steps: int, warmup: int) -> list[float]:
        """ms per call of `run()` (CUDA events), L2 flushed (256 MB memset) before each."""
        if self._flush is None:
            self._flush = self.d.alloc(256 << 20)
        for _ in range(warmup):
            run()
        self.d.sync()
        e0, e1 = self.d.event(), self.d.event()
        out = []
        for _ in range(steps):
            self.d.cu.cuMemsetD8_v2(self._flush, 0, 256 << 20)
            self.d.cu.cuEventRecord(e0, None)
            run()
            self.d.cu.cuEventRecord(e1, None)
            out.append(self.d.elapsed_ms(e0, e1))
        self.d.cu.cuEventDestroy_v2(e0)
        self.d.cu.cuEventDestroy_v2(e1)
        return out


def pairwise(a, b, k: int = -1, out8: bool = False, device: int = 0) -> np.ndarray:
    """d(a_i, b_i) by the reference's kernels (test helper)."""
    r = RefCuda(device)
    try:
        st = r.pairs_setup(a, b)
        n = st["n"]
        res = np.empty(n, np.uint8 if out8 else np.int32)
        out = r._keep(r.d.alloc(res.nbytes))
        r.pairs_run(st, out, k, out8)
        r.d.sync()
        return r.d.download(out, res)
    finally:
        r.close()


def cdist(q, c, k: int = -1, out8: bool = False, device: int = 0) -> np.ndarray:
    """d(q_i, c_j) by the reference's kernels (test helper)."""
    r = RefCuda(device)
    try:
        st = r.cross_setup(q, c)
        res = np.empty((st["nq"], st["nc"]), np.uint8 if out8 else np.int32)
        out = r._keep(r.d.alloc(res.nbytes))
        r.cross_run(st, out, k, out8)
        r.d.sync()
        return r.d.download(out, res)
    finally:
        r.close()
