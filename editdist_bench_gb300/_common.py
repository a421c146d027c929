"""Input checks, packing and output conversion with bitlev's semantics.

Mirrors bitlev/_common.py:9-33 (``check_k``, ``check_dtype``, ``convert``,
``as_list``) and the str/bytes rules of bitlev's C extension
(csrc/edpy.c:14-35, ``pack`` at :200-224), with the same exception types
and messages, so code written against ``bitlev.gpu`` sees the same errors.
"""
from __future__ import annotations

import numpy as np

DTYPES = (np.int32, np.uint16, np.uint8)
DTYPE_CODE = {np.dtype(np.int32): 0, np.dtype(np.uint16): 1, np.dtype(np.uint8): 2}
K_CLAMP = 2 ** 30

_WIDE_MSG = "string has characters above U+00FF; pass bytes (e.g. UTF-8 encoded) instead"
_TYPE_MSG = "expected str or bytes"


def check_k(max_dist) -> int:
    """None -> -1 (exact); negative -> ValueError; clamp to 2**30."""
    if max_dist is None:
        return -1
    k = int(max_dist)
    if k < 0:
        raise ValueError("max_dist must be >= 0 (or None)")
    return min(k, K_CLAMP)


def check_dtype(dtype) -> np.dtype:
    dt = np.dtype(dtype)
    if dt not in [np.dtype(d) for d in DTYPES]:
        raise ValueError("dtype must be numpy int32, uint16 or uint8")
    return dt


def convert(out: np.ndarray, dt) -> np.ndarray:
    """int32 -> requested dtype; narrower types saturate at their maximum."""
    if dt == np.int32:
        return out
    return np.minimum(out, np.iinfo(dt).max).astype(dt)


def as_list(x):
    return x if isinstance(x, list) else list(x)


def _encode_one(s) -> bytes:
    if isinstance(s, str):
        try:
            return s.encode("latin-1")
        except UnicodeEncodeError:
            raise ValueError(_WIDE_MSG) from None
    if isinstance(s, bytes):
        return s
    raise TypeError(_TYPE_MSG)


try:                                    # the native packer (csrc/blg_pack.c), when built
    from . import _blgpack
except ImportError:
    _blgpack = None


def pack(strings):
    """Packed (uint8 buffer, int64 offsets[n+1]) of a sequence of str/bytes:
    1 character = 1 byte, str must be Latin-1, the buffer is never empty.
    The native packer validates every item, then copies each string's bytes
    once; without it the bytes are joined by Python."""
    seq = as_list(strings)
    if _blgpack is not None:
        n, total = _blgpack.size(seq)
        buf = np.empty(max(total, 1), dtype=np.uint8)
        off = np.empty(n + 1, dtype=np.int64)
        _blgpack.pack_into(seq, buf.ctypes.data, buf.size, off.ctypes.data)
        return buf, off
    return pack_python(seq)


def pack_python(strings):
    """pack() in Python: one join of the str or bytes items."""
    seq = as_list(strings)
    n = len(seq)
    off = np.zeros(n + 1, dtype=np.int64)
    if n == 0:
        return np.zeros(1, dtype=np.uint8), off
    first = seq[0]
    raw = None
    if isinstance(first, str):
        try:
            joined = "".join(seq)                   # TypeError when an item is not str
        except TypeError:
            joined = None
        if joined is not None:
            try:
                raw = joined.encode("latin-1")
            except UnicodeEncodeError:
                raise ValueError(_WIDE_MSG) from None
    elif isinstance(first, bytes) and all(isinstance(s, bytes) for s in seq):
        raw = b"".join(seq)
    if raw is None:                                 # mixed str / bytes, or a bad item
        parts = [_encode_one(s) for s in seq]
        raw = b"".join(parts)
        lens = np.fromiter((len(p) for p in parts), dtype=np.int64, count=n)
    else:
        lens = np.fromiter(map(len, seq), dtype=np.int64, count=n)
    np.cumsum(lens, out=off[1:])
    buf = np.frombuffer(raw, dtype=np.uint8) if raw else np.zeros(1, dtype=np.uint8)
    return buf, off
