"""A minimal device array for ``return_device=True`` results.

The reference returns a CuPy ndarray (bitlev/gpu.py:64-68). Without CuPy,
results stay in HBM in a buffer owned by the library and are exposed through
``__cuda_array_interface__`` (version 3), so CuPy, Numba or PyTorch can wrap
them without a copy; ``get()`` copies to a numpy array like ``cupy.ndarray.get``.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib


class DeviceArray:
    __slots__ = ("_ptr", "shape", "dtype", "_ctx", "_owner", "__weakref__")

    def __init__(self, ptr: int, shape, dtype, ctx: "_lib.Context", owner=None):
        self._ptr = int(ptr or 0)
        self.shape = tuple(int(s) for s in shape)
        self.dtype = np.dtype(dtype)
        self._ctx = ctx
        self._owner = owner          # None: this object frees the buffer

    # ---- array protocol --------------------------------------------------
    @property
    def __cuda_array_interface__(self):
        return {"shape": self.shape, "typestr": self.dtype.str, "data": (self._ptr, False),
                "version": 3, "strides": None, "stream": None}

    @property
    def ptr(self) -> int:
        return self._ptr

    @property
    def size(self) -> int:
        n = 1
        for s in self.shape:
            n *= s
        return n

    @property
    def ndim(self) -> int:
        return len(self.shape)

    @property
    def nbytes(self) -> int:
        return self.size * self.dtype.itemsize

    def __len__(self):
        if not self.shape:
            raise TypeError("len() of a 0-d array")
        return self.shape[0]

    def get(self) -> np.ndarray:
        """Copy to a host numpy array."""
        out = np.empty(self.shape, dtype=self.dtype)
        if self.nbytes:
            self._ctx.check(self._ctx.lib.blg_memcpy_d2h(self._ctx.h, out.ctypes.data, self._ptr,
                                                         ctypes.c_size_t(self.nbytes)), "D2H")
        return out

    def tolist(self):
        return self.get().tolist()

    def reshape(self, *shape) -> "DeviceArray":
        if len(shape) == 1 and isinstance(shape[0], (tuple, list)):
            shape = tuple(shape[0])
        shape = list(shape)
        if shape.count(-1) > 1:
            raise ValueError("can only specify one unknown dimension")
        if -1 in shape:
            rest = 1
            for s in shape:
                if s != -1:
                    rest *= s
            shape[shape.index(-1)] = self.size // rest if rest else 0
        n = 1
        for s in shape:
            n *= s
        if n != self.size:
            raise ValueError(f"cannot reshape array of size {self.size} into shape {tuple(shape)}")
        return DeviceArray(self._ptr, shape, self.dtype, self._ctx, owner=self._owner or self)

    def __repr__(self):
        return f"DeviceArray(shape={self.shape}, dtype={self.dtype}, ptr=0x{self._ptr:x})"

    def __del__(self):
        if self._owner is None and self._ptr and self._ctx is not None and self._ctx.h:
            try:
                self._ctx.lib.blg_free(self._ctx.h, self._ptr)
            except Exception:
                pass
            self._ptr = 0
