"""The exact search over lexicographically sorted choices with column-state
reuse across shared prefixes (k_search_pfx): every result equals the oracle,
with choices built to share prefixes of every length (stems plus random
tails), duplicates, empty and very short choices, choices longer than the
checkpoint columns and than 255 bytes, partial tiles, partial query groups,
and queries of one and two 64-bit words. The launch labels confirm the
prefix kernel ran."""
import ctypes

import numpy as np
import pytest

import oracle
from editdist_bench_gb300 import _lib, workloads as W

pytestmark = pytest.mark.gpu


def _labels(ctx, fn):
    ctx.check(ctx.lib.blg_profile_enable(ctx.h, 1))
    try:
        fn()
    finally:
        buf = ctypes.create_string_buffer(8192)
        ctx.check(ctx.lib.blg_profile_report(ctx.h, buf, 8192))
        ctx.check(ctx.lib.blg_profile_enable(ctx.h, 0))
    return {line.split()[0] for line in buf.value.decode().splitlines()}


def _stemmed_choices(rng, n, stems, max_tail, alphabet=W.DNA):
    """n choices = a random stem (shared prefix source) cut at a random
    length, plus a random tail: sorted neighbours share prefixes of every
    length."""
    st = W.random_strings(rng, rng.integers(0, 90, stems), alphabet)
    pick = rng.integers(0, stems, n)
    sl = np.diff(st[1])[pick]
    cutlen = (rng.random(n) * (sl + 1)).astype(np.int64)
    heads = W.take(st, pick)
    hb, ho = heads
    lens = cutlen
    off = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(lens, out=off[1:])
    src = np.repeat(ho[:-1], lens) + (np.arange(int(off[-1])) - np.repeat(off[:-1], lens))
    cut = (hb[src] if len(src) else np.zeros(1, np.uint8), off)
    tails = W.random_strings(rng, rng.integers(0, max_tail + 1, n), alphabet)
    a, b = cut, tails
    la, lb = np.diff(a[1]), np.diff(b[1])
    off2 = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(la + lb, out=off2[1:])
    buf = np.empty(max(1, int(off2[-1])), dtype=np.uint8)
    for i in range(n):                      # interleave head and tail per choice
        o = off2[i]
        buf[o:o + la[i]] = a[0][a[1][i]:a[1][i + 1]]
        buf[o + la[i]:o + la[i] + lb[i]] = b[0][b[1][i]:b[1][i + 1]]
    return buf, off2


@pytest.mark.parametrize("seed", [1, 2])
def test_prefix_search_matches_oracle(gpu, seed):
    rng = np.random.default_rng(300 + seed)
    c = _stemmed_choices(rng, 9001, 40, 30)
    # duplicates, empty and very short choices, long ones (> 64 and > 255 bytes)
    extra = W.concat(W.take(c, rng.integers(0, 9001, 200)), W.random_strings(rng, [0, 0, 1, 2, 3, 5, 7]),
                     W.random_strings(rng, rng.integers(65, 300, 40)))
    c = W.take(W.concat(c, extra), rng.permutation(9001 + 247))
    q = W.concat(W.random_strings(rng, rng.integers(0, 129, 35)), W.random_strings(rng, [0, 1, 64, 65, 128]),
                 W.take(c, rng.integers(0, 9248, 6)))
    want = oracle.cross(q, c, threads=8)
    ctx = _lib.context()
    s = gpu.SearchBatch(q, c)
    out = s.alloc("int32")
    labels = _labels(ctx, lambda: s.run(out))
    assert "search_pfx" in labels, labels
    np.testing.assert_array_equal(out.get(), want)
    for dt in ("uint8", "uint16"):             # narrow stores through the permutation
        np.testing.assert_array_equal(s.run(s.alloc(dt)).get(), oracle.saturate(want, dt))
    # the one-call path builds the same layout
    np.testing.assert_array_equal(gpu.cdist_packed(q, c), want)


def test_prefix_search_benchmark_shape_rows(gpu):
    """The benchmark's own shape (length 64 DNA, 1% planted mutants) at a
    reduced query count: the prefix kernel runs and agrees with the oracle."""
    w = W.config2(nq=64, nc=65536, seed=77)
    ctx = _lib.context()
    s = gpu.SearchBatch(w.q, w.c)
    out = s.alloc("int32")
    labels = _labels(ctx, lambda: s.run(out))
    assert "search_pfx" in labels, labels
    rows = np.arange(0, 64, 5)
    np.testing.assert_array_equal(out.get()[rows], oracle.cross(W.take(w.q, rows), w.c, threads=8))
