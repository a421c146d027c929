"""Failure paths, made on the host: no test here faults, traps or hangs a GPU.

* An injected allocation failure (blg_set_fault_injection) at each device
  allocation of a one-call pairwise / cdist / matches-only cdist in turn
  raises MemoryError, and
  the next call on the same context is correct. The reference's error model
  is the same: an allocation failure returns -1 / raises MemoryError
  (csrc/myers.c:162-164, bench/cmyers.py:82-84).
* The short-pair tile kernel's bounded wait for its staged strings, cut to
  zero polls, ends the call with the timeout status (RuntimeError); the
  kernel still waits for its copies in flight, and the context stays usable.
"""
import numpy as np
import pytest

import oracle
from editdist_bench_gb300 import _lib, workloads as W

pytestmark = pytest.mark.gpu


def _inject(ctx, alloc_fail_after=-1, wait_polls=-1):
    ctx.check(ctx.lib.blg_set_fault_injection(ctx.h, alloc_fail_after, wait_polls))


def _sweep_allocations(gpu, call, check, limit=80):
    """Fail the 1st, 2nd, ... allocation of `call` until it needs fewer;
    after every injected failure the same call without injection is right."""
    ctx = _lib.context()
    failed = 0
    try:
        for after in range(limit):
            _inject(ctx, alloc_fail_after=after)
            try:
                got = call()
            except MemoryError:
                failed += 1
                _inject(ctx)
                check(call())
                continue
            _inject(ctx)
            check(got)
            break
        else:
            pytest.fail(f"call still allocating after {limit} allocations")
    finally:
        _inject(ctx)
    assert failed >= 1, "no allocation was failed"
    return failed


def test_alloc_failure_pairwise_paths(gpu):
    rng = np.random.default_rng(41)
    # mixed lengths (scheduled path, long patterns over lanes)
    a = W.random_strings(rng, rng.integers(0, 300, 1500))
    b = W.mutate(rng, a, 0.1)
    want = oracle.pairs(a, b, 8)
    n1 = _sweep_allocations(gpu, lambda: gpu.pairwise_packed(a, b, max_dist=8, dtype=np.uint8),
                            lambda got: np.testing.assert_array_equal(got, oracle.saturate(want, "uint8")))
    # short pairs (tile kernel); exact
    w = W.config1(n=4096, seed=12)
    want1 = oracle.pairs(w.a, w.b)
    n2 = _sweep_allocations(gpu, lambda: gpu.pairwise_packed(w.a, w.b),
                            lambda got: np.testing.assert_array_equal(got, want1))
    # the pipelined one-call path (2^18 pairs: chunked copies on two streams)
    w3 = W.config1(n=1 << 18, seed=13)
    want3 = oracle.pairs(w3.a, w3.b)
    n3 = _sweep_allocations(gpu, lambda: gpu.pairwise_packed(w3.a, w3.b),
                            lambda got: np.testing.assert_array_equal(got, want3))
    assert min(n1, n2, n3) >= 1


def test_alloc_failure_cdist_paths(gpu):
    rng = np.random.default_rng(42)
    q = W.random_strings(rng, rng.integers(0, 200, 40))
    c = W.concat(W.mutate(rng, q, 0.05), W.random_strings(rng, rng.integers(0, 200, 600)))
    for k, dt in ((None, "int32"), (3, "uint8")):
        want = oracle.saturate(oracle.cross(q, c, k), dt)
        _sweep_allocations(gpu, lambda: gpu.cdist_packed(q, c, max_dist=k, dtype=dt),
                           lambda got: np.testing.assert_array_equal(got, want))
    # the pipelined one-call path (a 64 MiB int32 matrix: query chunks with
    # their rows copied back while the next chunk computes); 4 rows checked
    w = W.config2(nq=256, nc=65536, seed=14)
    rows = np.arange(0, 256, 64)
    want = oracle.cross(W.take(w.q, rows), w.c)
    _sweep_allocations(gpu, lambda: gpu.cdist_packed(w.q, w.c),
                       lambda got: np.testing.assert_array_equal(got[rows], want))


def test_alloc_failure_matches_paths(gpu):
    """The matches-only search from the survivor kernel's result list (the
    automatic schedule) and from the dense scratch (the plain one)."""
    rng = np.random.default_rng(43)
    q = W.random_strings(rng, rng.integers(0, 150, 30))
    c = W.concat(W.mutate(rng, W.take(q, rng.integers(0, 30, 200)), 0.05), W.random_strings(rng, rng.integers(0, 160, 700)))
    d = oracle.cross(q, c, 4)
    qi, ci = np.nonzero(d <= 4)

    def check(got):
        np.testing.assert_array_equal(got[0], qi)
        np.testing.assert_array_equal(got[1], ci)
        np.testing.assert_array_equal(got[2], d[qi, ci])

    for sched in ("auto", "plain"):
        gpu.set_schedule(sched)
        try:
            _sweep_allocations(gpu, lambda: gpu.cdist_matches_packed(q, c, 4), check)
        finally:
            gpu.set_schedule("auto")


def test_alloc_failure_resident_matches_keeps_search_whole(gpu, monkeypatch):
    """A resident search whose matches call walks query chunks (the dense
    path: plain schedule, a scratch budget of 4 rows) and fails at any of
    its allocations still holds every query afterwards: its class set is
    rebuilt for all rows whatever happened, so the next matches call and
    the next dense run are exact."""
    rng = np.random.default_rng(44)
    q = W.random_strings(rng, rng.integers(0, 120, 23))
    c = W.concat(W.mutate(rng, W.take(q, rng.integers(0, 23, 150)), 0.08), W.random_strings(rng, rng.integers(0, 130, 400)))
    nc = len(c[1]) - 1
    d = oracle.cross(q, c, 3)
    qi, ci = np.nonzero(d <= 3)
    dense = oracle.saturate(d, "uint8")
    monkeypatch.setenv("BLG_MATCH_SCRATCH_BYTES", str(4 * nc))
    gpu.set_schedule("plain")
    try:
        s = gpu.SearchBatch(q, c)
        out = s.alloc("uint8")

        def check(got):
            np.testing.assert_array_equal(got[0], qi)
            np.testing.assert_array_equal(got[1], ci)
            np.testing.assert_array_equal(got[2], d[qi, ci])
            np.testing.assert_array_equal(s.run(out, max_dist=3).get(), dense)

        _sweep_allocations(gpu, lambda: s.matches(3), check)
    finally:
        gpu.set_schedule("auto")


def test_tile_wait_timeout_is_reported_and_recoverable(gpu):
    ctx = _lib.context()
    w = W.config1(n=8192, seed=15)
    want = oracle.pairs(w.a, w.b)
    try:
        _inject(ctx, wait_polls=0)
        with pytest.raises(RuntimeError, match="timed out"):
            gpu.pairwise_packed(w.a, w.b)
    finally:
        _inject(ctx)
    np.testing.assert_array_equal(gpu.pairwise_packed(w.a, w.b), want)
    # a resident run after the timeout is right too
    batch = gpu.PairsBatch(w.a, w.b)
    out = batch.alloc("int32")
    batch.run(out)
    np.testing.assert_array_equal(out.get(), want)
