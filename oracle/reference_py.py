"""ORACLE — test infrastructure only (never imported by the product path).

Pure-Python restatement of the reference's two ground-truth algorithms
(karims/editdist-bench bench/reference.py):

* ``dp_distance``    — textbook Wagner-Fischer, two rows (bench/reference.py:16-28);
* ``myers_distance`` — Myers/Hyyro bit-parallel over Python big integers, any
  length, no word limit (bench/reference.py:31-67).

Both take ``str`` or ``bytes``; strings are compared code unit by code unit,
bytes byte by byte.  ``capped`` applies the max_dist rule min(d, k+1) of
bitlev (bitlev/_common.py:9-15; csrc/myers.c:101-106) and ``saturate`` the
narrow-dtype rule (bitlev/_common.py:25-29).  Only small cases use these
loops; the C restatement (myers_oracle.c) is the bulk oracle.
"""
from __future__ import annotations

import numpy as np


def dp_distance(a, b) -> int:
    """Unit-cost Levenshtein distance by the full O(|a||b|) recurrence."""
    if len(a) < len(b):
        a, b = b, a
    row = list(range(len(b) + 1))
    for i, ca in enumerate(a, 1):
        diag, row[0] = row[0], i
        for j, cb in enumerate(b, 1):
            up = row[j]
            row[j] = min(up + 1, row[j - 1] + 1, diag + (ca != cb))
            diag = up
    return row[-1]


def myers_distance(a, b) -> int:
    """Bit-parallel distance: pattern ``a`` in the bit vectors, text ``b``
    scanned left to right; ``score`` follows the last pattern row."""
    m = len(a)
    if m == 0:
        return len(b)
    full = (1 << m) - 1
    top = 1 << (m - 1)
    peq: dict = {}
    for i, ch in enumerate(a):
        peq[ch] = peq.get(ch, 0) | (1 << i)
    pv, mv, score = full, 0, m
    for ch in b:
        eq = peq.get(ch, 0)
        xv = eq | mv
        xh = ((((eq & pv) + pv) & full) ^ pv) | eq
        ph = mv | (~(xh | pv) & full)
        mh = pv & xh
        score += (1 if ph & top else 0) - (1 if mh & top else 0)
        ph = ((ph << 1) | 1) & full        # global alignment: +1 enters at the top row
        mh = (mh << 1) & full
        pv = mh | (~(xv | ph) & full)
        mv = ph & xv
    return score


def capped(d: int, max_dist) -> int:
    """bitlev's max_dist rule: None -> exact, k -> min(d, k + 1)."""
    return d if max_dist is None else min(d, int(max_dist) + 1)


def saturate(values, dtype) -> np.ndarray:
    """int results -> dtype, narrower types saturating at their maximum."""
    arr = np.asarray(values, dtype=np.int64)
    dt = np.dtype(dtype)
    if dt == np.int32:
        return arr.astype(np.int32)
    return np.minimum(arr, np.iinfo(dt).max).astype(dt)
