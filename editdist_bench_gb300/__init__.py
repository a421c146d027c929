"""editdist_bench_gb300 — a GB300-native engine for bitlev's GPU hot path.

Exact unit-cost Levenshtein distances (score only) for batches of byte
strings, computed by hand-written sm_103a CUDA kernels behind a C-ABI
(``libbitlev_gb300.so``, include/bitlev_gb300.h) that this package loads
through ctypes. ``editdist_bench_gb300.gpu`` is the drop-in for
``bitlev.gpu`` (bitlev/gpu.py): ``pairwise``, ``cdist``, ``available``.
"""
from __future__ import annotations

from . import gpu  # noqa: F401
from .device_array import DeviceArray  # noqa: F401

__version__ = "0.1.0"
__all__ = ["gpu", "DeviceArray"]
