"""Deferred banded survivors (thresholded search, max_dist <= 31): a job runs
each survivor for 4 (k + 4) columns and queues the ones still inside the
band; one resume launch finishes them from their saved column state. The
results equal the oracle and the undeferred run (capacity 0) whatever the
queue capacity: the default, and a capacity of a few items, where most
long survivors overflow the queue and finish inside their jobs. Covered:
the resident search (every query word class), the one-call pipeline, k = 0
and k = 31 (the longest first stretch, 140 columns), and the multi-problem
batch graph. Reference semantics: csrc/myers.c:101-143 (exit rules, caps)."""
import os

import numpy as np
import pytest

import oracle
from editdist_bench_gb300 import _lib, workloads as W

pytestmark = pytest.mark.gpu

THREADS = max(1, min(16, os.cpu_count() or 1))


def _cap(cap):
    ctx = _lib.context()
    ctx.check(ctx.lib.blg_set_defer_capacity(ctx.h, cap))


@pytest.fixture
def restore_cap():
    yield
    _cap(1 << 20)


def _near_copy_search(seed, nq, nc, lo, hi):
    """Queries of lengths lo..hi and choices of which a quarter are near-copies
    of a query (edit rates 0..6%), the rest random: many survivors run the
    whole text, so the queue fills."""
    rng = np.random.default_rng(seed)
    q = W.random_strings(rng, rng.integers(lo, hi + 1, nq))
    n_plant = nc // 4
    planted = W.mutate(rng, W.take(q, rng.integers(0, nq, n_plant)), rng.uniform(0.0, 0.06, n_plant))
    rest = W.random_strings(rng, rng.integers(lo, hi + 1, nc - n_plant))
    c = W.take(W.concat(planted, rest), rng.permutation(nc))
    return q, c


@pytest.mark.parametrize("k", [0, 4, 9, 31])
def test_defer_capacities_agree(gpu, restore_cap, k):
    q, c = _near_copy_search(800 + k, 96, 40000, 40, 256)
    s = gpu.SearchBatch(q, c)
    got = {}
    for cap in (1 << 20, 5, 0):
        _cap(cap)
        got[cap] = s.run(s.alloc("uint8"), max_dist=k).get()
    np.testing.assert_array_equal(got[5], got[0])
    np.testing.assert_array_equal(got[1 << 20], got[0])
    want = oracle.saturate(oracle.cross(q, c, k, threads=THREADS), "uint8")
    np.testing.assert_array_equal(got[1 << 20], want)
    assert (want <= k).sum() > 100                          # the near-copies are found


def test_defer_one_call_pipeline(gpu, restore_cap):
    q, c = _near_copy_search(811, 300, 70000, 60, 200)
    want = oracle.saturate(oracle.cross(q, c, 6, threads=THREADS), "uint16")
    for cap in (1 << 20, 3):
        _cap(cap)
        np.testing.assert_array_equal(gpu.cdist_packed(q, c, max_dist=6, dtype="uint16"), want, err_msg=str(cap))


def test_defer_batch_graph(gpu, restore_cap):
    rng = np.random.default_rng(820)
    probs = []
    for i in range(12):
        q, c = _near_copy_search(830 + i, int(rng.integers(1, 40)), int(rng.integers(500, 9000)), 16, 256)
        probs.append((q, c, int(rng.integers(0, 9)), ("uint8", "uint16", "int32")[i % 3]))
    probs.append((probs[0][0], probs[0][1], None, "int32"))       # an exact problem beside them
    outs = {}
    for cap in (1 << 20, 2, 0):
        _cap(cap)                                                  # a new graph captures the setting
        batch = gpu.ProblemBatch(probs)
        for _ in range(2):                                         # capture, then replay
            res = batch.run()
            gpu.synchronize()
            outs[cap] = [o.get() for o in res]
    for i, (q, c, k, dt) in enumerate(probs):
        want = oracle.saturate(oracle.cross(q, c, k, threads=THREADS), dt)
        for cap, o in outs.items():
            np.testing.assert_array_equal(o[i], want, err_msg=f"problem {i} capacity {cap}")


def test_defer_capacity_argument(gpu, restore_cap):
    ctx = _lib.context()
    assert ctx.lib.blg_set_defer_capacity(ctx.h, -1) == _lib.ERR_ARG
    ctx.check(ctx.lib.blg_set_defer_capacity(ctx.h, 1 << 30))     # clamped to the queue's size
