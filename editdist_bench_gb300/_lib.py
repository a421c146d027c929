"""ctypes binding of ``libbitlev_gb300.so`` (declared in include/bitlev_gb300.h).

The library is built in-tree by ``editdist_bench_gb300._build.build()``. There
is no fallback: when the library is missing or no GPU is visible the calls
raise, exactly where the reference would fail to import CuPy or find a device.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

from . import _build

OK, ERR_ALLOC, ERR_ARG, ERR_CUDA, ERR_TIMEOUT, ERR_NODEVICE = 0, -1, -2, -3, -4, -5
SCHED_AUTO, SCHED_PLAIN, SCHED_LEARNED, SCHED_LENSORT = 0, 1, 2, 3
UINT4 = 3            # BLG_UINT4: 4-bit results, two per byte

_P = ctypes.c_void_p
_I32, _I64, _SZ = ctypes.c_int32, ctypes.c_int64, ctypes.c_size_t

# (name, restype, argtypes) of every symbol in include/bitlev_gb300.h
SIGNATURES = [
    ("blg_version", ctypes.c_int, []),
    ("blg_device_count", ctypes.c_int, []),
    ("blg_init", ctypes.c_int, [ctypes.c_int, ctypes.POINTER(_P)]),
    ("blg_destroy", None, [_P]),
    ("blg_last_error", ctypes.c_char_p, [_P]),
    ("blg_pairwise", ctypes.c_int, [_P, _P, _P, _P, _P, _I64, _I32, _I32, _P, ctypes.POINTER(_P)]),
    ("blg_cdist", ctypes.c_int, [_P, _P, _P, _I64, _P, _P, _I64, _I32, _I32, _P, ctypes.POINTER(_P)]),
    ("blg_pairs_upload", ctypes.c_int, [_P, _P, _P, _P, _P, _I64, ctypes.POINTER(_P)]),
    ("blg_pairs_run", ctypes.c_int, [_P, _P, _I32, _I32, _P]),
    ("blg_pairs_free", None, [_P, _P]),
    ("blg_pairs_run_logged", ctypes.c_int, [_P, _P, _I32, _I32, _P, _P]),
    ("blg_search_upload", ctypes.c_int, [_P, _P, _P, _I64, _P, _P, _I64, ctypes.POINTER(_P)]),
    ("blg_search_run", ctypes.c_int, [_P, _P, _I32, _I32, _P]),
    ("blg_search_free", None, [_P, _P]),
    ("blg_batch_upload", ctypes.c_int, [_P, _P, _I32, ctypes.POINTER(_P)]),
    ("blg_batch_run", ctypes.c_int, [_P, _P]),
    ("blg_batch_pairs", _I64, [_P]),
    ("blg_batch_free", None, [_P, _P]),
    ("blg_cdist_batch", ctypes.c_int, [_P, _P, _I32]),
    ("blg_cdist_noalloc", ctypes.c_int, [_P, _P, _SZ, _P, _I64, _P, _SZ, _P, _I64, _I32, _I32, _P]),
    ("blg_sched_train", ctypes.c_int, [_P, _P, _I32, _I32, ctypes.c_float, _I64, ctypes.POINTER(ctypes.c_float)]),
    ("blg_sched_train_search", ctypes.c_int, [_P, _P, _I32, _I32, ctypes.c_float, _I64,
                                              ctypes.POINTER(ctypes.c_float)]),
    ("blg_sched_set_weights", ctypes.c_int, [_P, _P, ctypes.c_int]),
    ("blg_sched_get_weights", ctypes.c_int, [_P, _P, ctypes.c_int]),
    ("blg_sched_gradient", ctypes.c_int, [_P, _P, _P, ctypes.c_int, _P, ctypes.POINTER(ctypes.c_float)]),
    ("blg_sched_predict", ctypes.c_int, [_P, _P, _I64, _P]),
    ("blg_sched_save", ctypes.c_int, [_P, ctypes.c_char_p]),
    ("blg_sched_load", ctypes.c_int, [_P, ctypes.c_char_p]),
    ("blg_malloc", ctypes.c_int, [_P, _SZ, ctypes.POINTER(_P)]),
    ("blg_free", ctypes.c_int, [_P, _P]),
    ("blg_cdist_matches", ctypes.c_int, [_P, _P, _P, _I64, _P, _P, _I64, _I32, _P, _I64, ctypes.POINTER(_I64)]),
    ("blg_search_matches", ctypes.c_int, [_P, _P, _I32, _P, _I64, ctypes.POINTER(_I64)]),
    ("blg_host_alloc", ctypes.c_int, [_P, _SZ, ctypes.POINTER(_P)]),
    ("blg_host_free", ctypes.c_int, [_P, _P]),
    ("blg_memcpy_h2d", ctypes.c_int, [_P, _P, _P, _SZ]),
    ("blg_memcpy_d2h", ctypes.c_int, [_P, _P, _P, _SZ]),
    ("blg_memset", ctypes.c_int, [_P, _P, ctypes.c_int, _SZ]),
    ("blg_synchronize", ctypes.c_int, [_P]),
    ("blg_timer_start", ctypes.c_int, [_P]),
    ("blg_timer_stop", ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_float)]),
    ("blg_launch_count", ctypes.c_int64, [_P]),
    ("blg_set_schedule", ctypes.c_int, [_P, ctypes.c_int]),
    ("blg_autotune", ctypes.c_int, [_P, ctypes.c_char_p]),
    ("blg_get_tuning", ctypes.c_int, [_P, _P, ctypes.c_int]),
    ("blg_set_fault_injection", ctypes.c_int, [_P, _I64, _I32]),
    ("blg_profile_enable", ctypes.c_int, [_P, ctypes.c_int]),
    ("blg_profile_report", ctypes.c_int, [_P, ctypes.c_char_p, _SZ]),
]

class Problem(ctypes.Structure):
    """blg_problem (include/bitlev_gb300.h)."""
    _fields_ = [("buf_q", _P), ("off_q", _P), ("nq", _I64), ("buf_c", _P), ("off_c", _P), ("nc", _I64),
                ("max_dist", _I32), ("dtype", _I32), ("d_out", _P)]


_lib = None
_ctx = None
_lock = threading.Lock()


def library_path() -> str:
    return _build.LIB


def load(path: str | None = None):
    """Load the CUDA library and declare every exported signature."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or library_path()
    if not os.path.exists(p):
        raise ImportError(f"CUDA library not built: {p} (run __graft_entry__.build() or "
                          "python -m editdist_bench_gb300._build)")
    lib = ctypes.CDLL(p)
    for name, res, args in SIGNATURES:
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    if path is None:
        _lib = lib
    return lib


class Context:
    """One library context (device, stream, status word) for this process."""

    def __init__(self, device: int = 0):
        self.lib = load()
        h = _P()
        rc = self.lib.blg_init(int(device), ctypes.byref(h))
        if rc != OK:
            raise RuntimeError(f"blg_init({device}) failed with code {rc}"
                               + (": no CUDA device" if rc == ERR_NODEVICE else ""))
        self.h = h
        self.device = device

    def check(self, rc: int, what: str = ""):
        if rc == OK:
            return
        msg = (self.lib.blg_last_error(self.h) or b"").decode(errors="replace")
        text = f"{what}: {msg}" if what else msg
        if rc == ERR_ALLOC:
            raise MemoryError(text)
        if rc == ERR_ARG:
            raise ValueError(text)
        raise RuntimeError(f"{text} (code {rc})")

    def close(self):
        if getattr(self, "h", None):
            self.lib.blg_destroy(self.h)
            self.h = None


def context() -> Context:
    global _ctx
    with _lock:
        if _ctx is None:
            _ctx = Context(int(os.environ.get("BLG_DEVICE", "0")))
        return _ctx


def device_count() -> int:
    try:
        return int(load().blg_device_count())
    except (ImportError, OSError):
        return 0


def ptr(a: np.ndarray) -> int:
    return a.ctypes.data
