"""Resident pairs runs as one CUDA graph launch: the first run with a set of
parameters runs directly, the second is captured, later ones replay the
graph. Every run's results equal the oracle, through the tile path (short
pairs), the scheduled plan (uneven pairs, banded and full-word solvers) and
the natural-order schedule, across changes of max_dist, dtype, output
buffer and schedule that force a new capture."""
import numpy as np
import pytest

import oracle
from editdist_bench_gb300 import _lib, workloads as W

pytestmark = pytest.mark.gpu


def _runs(gpu, batch, cases, want_fn, repeats=4):
    for k, dt in cases:
        want = oracle.saturate(want_fn(k), dt)
        out = batch.alloc(dt)
        for r in range(repeats):
            batch.run(out, max_dist=k)
            np.testing.assert_array_equal(out.get(), want, err_msg=f"k={k} {dt} run {r}")


def test_graph_replay_tile_and_scheduled_paths(gpu):
    w1 = W.config1(n=20000, seed=71)
    b1 = gpu.PairsBatch(w1.a, w1.b)
    _runs(gpu, b1, [(None, "int32"), (3, "uint8"), (None, "int32")], lambda k: oracle.pairs(w1.a, w1.b, k))
    w3 = W.config3(n=30000, seed=72)
    b3 = gpu.PairsBatch(w3.a, w3.b)
    _runs(gpu, b3, [(8, "uint8"), (31, "uint8"), (32, "uint16"), (None, "int32")],
          lambda k: oracle.pairs(w3.a, w3.b, k, threads=8))
    try:
        gpu.set_schedule("plain")
        _runs(gpu, b3, [(8, "uint8")], lambda k: oracle.pairs(w3.a, w3.b, k, threads=8))
    finally:
        gpu.set_schedule("auto")
    _runs(gpu, b3, [(8, "uint8")], lambda k: oracle.pairs(w3.a, w3.b, k, threads=8), repeats=2)


def test_graph_replay_counts_its_kernels(gpu):
    """A replayed run counts the kernels its graph holds."""
    ctx = _lib.context()
    w = W.config3(n=8000, seed=73)
    b = gpu.PairsBatch(w.a, w.b)
    out = b.alloc("uint8")
    counts = []
    for _ in range(4):
        c0 = ctx.lib.blg_launch_count(ctx.h)
        b.run(out, max_dist=8)
        counts.append(ctx.lib.blg_launch_count(ctx.h) - c0)
    gpu.synchronize()
    assert counts[0] == counts[1] == counts[2] == counts[3] > 0
    np.testing.assert_array_equal(out.get(), oracle.saturate(oracle.pairs(w.a, w.b, 8), "uint8"))
