"""Matches-only thresholded search (blg_cdist_matches / blg_search_matches):
the records are exactly the oracle's pairs with d <= max_dist, sorted by
(query, choice), with their distances; capacity truncation reports the full
count; both ways of finding them give the same records: the survivor
kernel's result list (max_dist <= 31 under the survivor schedules) and the
dense scratch compaction (max_dist > 31, the plain schedule, or a list that
ran full), the latter with every scratch width (uint8 / uint16 / int32 by
max_dist)."""
import numpy as np
import pytest

import oracle
from editdist_bench_gb300 import gpu, workloads as W

pytestmark = pytest.mark.gpu


def _want(q, c, k):
    d = oracle.cross(q, c, k)
    qi, ci = np.nonzero(d <= k)                 # row-major: sorted by (query, choice)
    return qi, ci, d[qi, ci]


def _check(got, want):
    for g, w, name in zip(got, want, ("query", "choice", "dist")):
        np.testing.assert_array_equal(np.asarray(g, dtype=np.int64), np.asarray(w, dtype=np.int64), err_msg=name)


@pytest.mark.parametrize("k", [0, 1, 3, 8, 31, 40])
def test_matches_equal_oracle(k):
    rng = np.random.default_rng(100 + k)
    q = W.random_strings(rng, rng.integers(0, 200, 37))
    c = W.concat(W.mutate(rng, W.take(q, rng.integers(0, 37, 300)), rng.uniform(0, 0.2, 300)),
                 W.random_strings(rng, rng.integers(0, 220, 900)))
    want = _want(q, c, k)
    assert len(want[0]) > 0
    _check(gpu.cdist_matches_packed(q, c, k), want)
    s = gpu.SearchBatch(q, c)
    _check(s.matches(k), want)


def test_matches_config4_shape():
    w = W.config4(nq=48, nc=1 << 15, seed=9)
    want = _want(w.q, w.c, 4)
    _check(gpu.cdist_matches_packed(w.q, w.c, 4), want)


@pytest.mark.parametrize("k", [300, 70000])
def test_matches_wide_thresholds(k):
    """k > 254 uses a uint16 scratch, k > 65534 an int32 one."""
    rng = np.random.default_rng(7)
    q = W.random_strings(rng, rng.integers(0, 400, 9))
    c = W.random_strings(rng, rng.integers(0, 700, 200))
    _check(gpu.cdist_matches_packed(q, c, k), _want(q, c, k))


def test_matches_capacity_reports_total():
    rng = np.random.default_rng(8)
    q = W.random_strings(rng, rng.integers(1, 40, 20))
    c = W.concat(q, W.mutate(rng, q, 0.1))
    want = _want(q, c, 5)
    n = len(want[0])
    assert n > 10
    part = gpu.cdist_matches_packed(q, c, 5, capacity=7)
    _check(part, tuple(x[:7] for x in want))
    s = gpu.SearchBatch(q, c)
    buf = s.match_buffer(5)
    assert s.matches_into(buf, 5) == n
    rec = buf.get()
    np.testing.assert_array_equal(rec["query"], want[0][:5])
    np.testing.assert_array_equal(rec["choice"], want[1][:5])


@pytest.mark.parametrize("sched", ["auto", "plain", "learned"])
def test_matches_every_schedule(sched):
    w = W.config4(nq=16, nc=1 << 13, seed=10)
    want = _want(w.q, w.c, 4)
    gpu.set_schedule(sched)
    try:
        _check(gpu.cdist_matches_packed(w.q, w.c, 4), want)
    finally:
        gpu.set_schedule("auto")


def test_matches_edges():
    rng = np.random.default_rng(11)
    q = W.random_strings(rng, np.array([0, 0, 3]))
    c = W.random_strings(rng, np.array([0, 1, 2, 5]))
    _check(gpu.cdist_matches_packed(q, c, 2), _want(q, c, 2))
    empty = W.random_strings(rng, np.array([], dtype=np.int64))
    got = gpu.cdist_matches_packed(empty, c, 2)
    assert all(len(x) == 0 for x in got)
    with pytest.raises(ValueError):
        gpu.cdist_matches_packed(q, c, None)


def test_matches_in_query_chunks(monkeypatch):
    """Under the plain schedule (the dense path), a small scratch budget
    (BLG_MATCH_SCRATCH_BYTES) makes both entry points walk several query
    chunks; the records are the same, and the resident search still runs
    dense afterwards (its classes are rebuilt)."""
    rng = np.random.default_rng(13)
    q = W.random_strings(rng, rng.integers(0, 120, 41))
    c = W.concat(W.mutate(rng, W.take(q, rng.integers(0, 41, 500)), 0.1), W.random_strings(rng, rng.integers(0, 130, 2500)))
    nc = len(c[1]) - 1
    want = _want(q, c, 3)
    monkeypatch.setenv("BLG_MATCH_SCRATCH_BYTES", str(5 * nc))      # 5 rows of uint8 per chunk
    gpu.set_schedule("plain")
    try:
        _check(gpu.cdist_matches_packed(q, c, 3), want)
        s = gpu.SearchBatch(q, c)
        _check(s.matches(3), want)
        out = s.alloc("uint8")
        np.testing.assert_array_equal(s.run(out, max_dist=3).get(), oracle.saturate(oracle.cross(q, c, 3), "uint8"))
    finally:
        gpu.set_schedule("auto")
    # the same search under the survivor schedule takes the result list
    _check(gpu.cdist_matches_packed(q, c, 3), want)
    _check(gpu.SearchBatch(q, c).matches(3), want)


def test_matches_list_full_falls_back():
    """More matches than the survivor kernel's result list holds (2^20
    entries): 1100 x 1000 equal strings at max_dist 0 are 1.1 M matches, so
    both entry points fall back to the dense path and still return every
    record."""
    rng = np.random.default_rng(14)
    one = W.random_strings(rng, np.array([6]))
    q, c = W.take(one, np.zeros(1100, dtype=np.int64)), W.take(one, np.zeros(1000, dtype=np.int64))
    qi, ci = np.divmod(np.arange(1100 * 1000, dtype=np.int64), 1000)
    want = (qi, ci, np.zeros(1100 * 1000, dtype=np.int64))
    assert len(qi) > (1 << 20)
    _check(gpu.cdist_matches_packed(q, c, 0, capacity=1100 * 1000), want)
    s = gpu.SearchBatch(q, c)
    _check(s.matches(0), want)
