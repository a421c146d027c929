"""ORACLE — test infrastructure only.

The CPU checker for the GPU hot path: a C restatement of bitlev's scalar
Myers core (myers_oracle.c, loaded here through ctypes), the pure-Python
ground truth (reference_py.py) and loaders for the reference's own CPU code
compiled from its sources (oracle/_ref, built by build_oracle.build_ref when
the reference checkout is present).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline legs
may import this package. The product package never does.
"""
from __future__ import annotations

import ctypes
import importlib.machinery
import importlib.util
import os
import sys

import numpy as np

from . import build_oracle
from .reference_py import capped, dp_distance, myers_distance, saturate  # noqa: F401

_P_U8 = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
_P_I64 = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
_P_I32 = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_LIB = None


def lib():
    """ctypes handle of oracle/_build/liborc.so (compiled on first use)."""
    global _LIB
    if _LIB is None:
        L = ctypes.CDLL(build_oracle.build_oracle())
        L.orc_pairs.argtypes = [_P_U8, _P_I64, _P_U8, _P_I64, ctypes.c_int64, ctypes.c_int32,
                                ctypes.c_int32, _P_I32]
        L.orc_pairs_trace.argtypes = L.orc_pairs.argtypes + [_P_I32, _P_I32, _P_I32]
        L.orc_pairs_mt.argtypes = L.orc_pairs.argtypes + [ctypes.c_int32]
        L.orc_cross.argtypes = [_P_U8, _P_I64, ctypes.c_int64, _P_U8, _P_I64, ctypes.c_int64,
                                ctypes.c_int32, _P_I32]
        L.orc_cross_trace.argtypes = L.orc_cross.argtypes + [_P_I32]
        L.orc_cross_mt.argtypes = L.orc_cross.argtypes + [ctypes.c_int32]
        for f in (L.orc_pairs, L.orc_pairs_trace, L.orc_pairs_mt, L.orc_cross,
                  L.orc_cross_trace, L.orc_cross_mt):
            f.restype = ctypes.c_int
        _LIB = L
    return _LIB


def pack(strings):
    """(uint8 buffer, int64 offsets[n+1]) — the layout of bitlev's
    ``_edpy.pack`` (csrc/edpy.c:200-224): strings concatenated, 1 char =
    1 byte (str must be Latin-1), buffer never empty."""
    enc = [s.encode("latin-1") if isinstance(s, str) else bytes(s) for s in strings]
    off = np.zeros(len(enc) + 1, dtype=np.int64)
    if enc:
        np.cumsum([len(e) for e in enc], out=off[1:])
    buf = np.frombuffer(b"".join(enc) or b"\0", dtype=np.uint8).copy()
    return buf, off


def _k(max_dist) -> int:
    return -1 if max_dist is None else min(int(max_dist), 2 ** 30)


def pairs(pa, pb, max_dist=None, trim=True, threads=1) -> np.ndarray:
    (ba, oa), (bb, ob) = pa, pb
    n = len(oa) - 1
    out = np.empty(n, dtype=np.int32)
    if threads > 1:
        rc = lib().orc_pairs_mt(ba, oa, bb, ob, n, _k(max_dist), int(trim), out, int(threads))
    else:
        rc = lib().orc_pairs(ba, oa, bb, ob, n, _k(max_dist), int(trim), out)
    if rc:
        raise MemoryError("oracle workspace allocation failed")
    return out


def pairs_trace(pa, pb, max_dist=None, trim=True):
    """(distances, trimmed pattern length m', text length n', columns processed)."""
    (ba, oa), (bb, ob) = pa, pb
    n = len(oa) - 1
    out, m_, n_, c_ = (np.empty(n, dtype=np.int32) for _ in range(4))
    if lib().orc_pairs_trace(ba, oa, bb, ob, n, _k(max_dist), int(trim), out, m_, n_, c_):
        raise MemoryError("oracle workspace allocation failed")
    return out, m_, n_, c_


def cross(pq, pc, max_dist=None, threads=1) -> np.ndarray:
    (bq, oq), (bc, oc) = pq, pc
    nq, nc = len(oq) - 1, len(oc) - 1
    out = np.empty(nq * nc, dtype=np.int32)
    if threads > 1:
        rc = lib().orc_cross_mt(bq, oq, nq, bc, oc, nc, _k(max_dist), out, int(threads))
    else:
        rc = lib().orc_cross(bq, oq, nq, bc, oc, nc, _k(max_dist), out)
    if rc:
        raise MemoryError("oracle workspace allocation failed")
    return out.reshape(nq, nc)


def cross_trace(pq, pc, max_dist=None):
    (bq, oq), (bc, oc) = pq, pc
    nq, nc = len(oq) - 1, len(oc) - 1
    out = np.empty(nq * nc, dtype=np.int32)
    cols = np.empty(nq * nc, dtype=np.int32)
    if lib().orc_cross_trace(bq, oq, nq, bc, oc, nc, _k(max_dist), out, cols):
        raise MemoryError("oracle workspace allocation failed")
    return out.reshape(nq, nc), cols.reshape(nq, nc)


def pairwise_api(a, b, max_dist=None, dtype=np.int32) -> np.ndarray:
    """Expected result of bitlev.pairwise / bitlev.gpu.pairwise."""
    return saturate(pairs(pack(a), pack(b), max_dist), dtype)


def cdist_api(q, c, max_dist=None, dtype=np.int32) -> np.ndarray:
    """Expected result of bitlev.cdist / bitlev.gpu.cdist."""
    return saturate(cross(pack(q), pack(c), max_dist), dtype)


# ---- the reference's own CPU code, compiled from its sources (here only) ----
def ref_built() -> bool:
    p = build_oracle.ref_paths()
    return all(os.path.exists(v) for v in p.values())


def ref_bitlev():
    """Import the reference's bitlev CPU package from the reference checkout,
    with its ``_edpy`` extension taken from oracle/_ref (the checkout is
    read-only, so the extension cannot sit beside it)."""
    if "bitlev" in sys.modules and getattr(sys.modules["bitlev"], "_BLG_REF", False):
        return sys.modules["bitlev"]
    paths = build_oracle.ref_paths()
    pkg_dir = os.path.join(build_oracle.REF_SRC, "bitlev")
    loader = importlib.machinery.ExtensionFileLoader("bitlev._edpy", paths["edpy"])
    spec = importlib.util.spec_from_file_location("bitlev._edpy", paths["edpy"], loader=loader)
    edpy = importlib.util.module_from_spec(spec)
    loader.exec_module(edpy)
    sys.modules["bitlev._edpy"] = edpy
    pspec = importlib.util.spec_from_file_location(
        "bitlev", os.path.join(pkg_dir, "__init__.py"), submodule_search_locations=[pkg_dir])
    mod = importlib.util.module_from_spec(pspec)
    sys.modules["bitlev"] = mod
    pspec.loader.exec_module(mod)
    mod._BLG_REF = True
    return mod


def ref_libmyers():
    """ctypes handle of the reference's libmyers.so (ed_pairs_k, ed_cross, ...)."""
    L = ctypes.CDLL(build_oracle.ref_paths()["libmyers"])
    L.ed_pairs_k.argtypes = [_P_U8, _P_I64, _P_U8, _P_I64, ctypes.c_int64, _P_I32,
                             ctypes.c_int, ctypes.c_int]
    L.ed_pairs_k.restype = ctypes.c_int
    L.ed_pairs_opt.argtypes = [_P_U8, _P_I64, _P_U8, _P_I64, ctypes.c_int64, _P_I32, ctypes.c_int]
    L.ed_pairs_opt.restype = ctypes.c_int
    L.ed_cross.argtypes = [_P_U8, _P_I64, ctypes.c_int64, _P_U8, _P_I64, ctypes.c_int64, _P_I32]
    L.ed_cross.restype = ctypes.c_int
    return L


def ref_gpucheck():
    """ctypes handle of the reference's host build of its GPU device functions."""
    L = ctypes.CDLL(build_oracle.ref_paths()["gpucheck"])
    L.gpu_pair_distance_host.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_char_p,
                                         ctypes.c_int, ctypes.c_int, ctypes.c_int]
    L.gpu_pair_distance_host.restype = ctypes.c_int
    L.gpu_peq_distance_host.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_char_p,
                                        ctypes.c_int, ctypes.c_int]
    L.gpu_peq_distance_host.restype = ctypes.c_int
    L.gpu_store8_host.argtypes = [ctypes.c_int]
    L.gpu_store8_host.restype = ctypes.c_int
    return L
