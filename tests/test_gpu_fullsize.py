"""GPU parity at the benchmark configurations' full sizes, where the kernel
plans differ from small cases (survivor job sizing and halving, query
chunking of the one-call pipelines, the 256-problem graph):

* thresholded search, 1024 x 2^20 choices, max_dist 4, uint8: sampled rows
  against the oracle, and the whole matrix under every work order and
  through the one-call pipeline equal to each other;
* the 256-problem batch at full scale through its captured graph: up to 4
  rows of every problem against the oracle, on the capture and a replay;
* the scheduled pairs path at the uneven-pairs configuration's lengths with
  max_dist 31 (banded solver) and 32 (full-word solver): every pair.

Reference semantics: csrc/myers.c:101-143 (exit rules and caps),
csrc/gpu_kernels.cu:53 (empty query), bitlev/_common.py:25-29 (saturation).
"""
import ctypes
import os

import numpy as np
import pytest

import oracle
from editdist_bench_gb300 import _lib, workloads as W

pytestmark = pytest.mark.gpu

THREADS = max(1, min(16, os.cpu_count() or 1))


def _rows(out, rows):
    """Rows of a device matrix, copied back one row at a time."""
    ctx = _lib.context()
    nq, nc = out.shape
    item = out.dtype.itemsize
    got = np.empty((len(rows), nc), dtype=out.dtype)
    for i, r in enumerate(rows):
        if nc:
            ctx.check(ctx.lib.blg_memcpy_d2h(ctx.h, got[i].ctypes.data, out.ptr + int(r) * nc * item, nc * item))
    return got


def test_config4_full_every_schedule(gpu):
    w = W.config4()
    s = gpu.SearchBatch(w.q, w.c)
    auto = s.run(s.alloc("uint8"), max_dist=4).get()
    rows = np.random.default_rng(4).choice(w.nq, 16, replace=False)
    want = oracle.saturate(oracle.cross(W.take(w.q, rows), w.c, 4, threads=THREADS), "uint8")
    np.testing.assert_array_equal(auto[rows], want)
    # the planted mutants are found: some pairs within max_dist in most rows
    assert (auto <= 4).any(axis=1).mean() > 0.5
    try:
        for sched in ("plain", "lensort"):
            gpu.set_schedule(sched)
            got = s.run(s.alloc("uint8"), max_dist=4).get()
            np.testing.assert_array_equal(got, auto, err_msg=sched)
            del got
    finally:
        gpu.set_schedule("auto")
    # the one-call pipeline (query chunks, rows copied back while the next chunk runs)
    np.testing.assert_array_equal(gpu.cdist_packed(w.q, w.c, max_dist=4, dtype="uint8"), auto)


def test_config5_full_graph(gpu):
    probs = W.config5()
    batch = gpu.ProblemBatch([(p.q, p.c, p.max_dist, p.dtype) for p in probs])
    rng = np.random.default_rng(5)
    for rep in range(2):                                  # capture, then replay
        outs = batch.run()
        gpu.synchronize()
        for i, (p, o) in enumerate(zip(probs, outs)):
            rows = np.sort(rng.choice(p.nq, min(4, p.nq), replace=False))
            want = oracle.saturate(oracle.cross(W.take(p.q, rows), p.c, p.max_dist, threads=THREADS), p.dtype)
            np.testing.assert_array_equal(_rows(o, rows), want, err_msg=f"problem {i} (pass {rep})")


@pytest.mark.parametrize("sched", ["auto", "plain"])
def test_scheduled_pairs_band_switch(gpu, sched):
    """max_dist 31 is the widest band the one-word banded solver takes; 32
    runs the full-word solvers. Lengths and edit rates of the uneven-pairs
    configuration (8..256 bytes, {A,C,G,T,N}, 0..30% edits)."""
    w = W.config3(n=1 << 18, seed=2031)
    gpu.set_schedule(sched)
    try:
        for k in (31, 32):
            want = oracle.saturate(oracle.pairs(w.a, w.b, k, threads=THREADS), "uint8")
            got = gpu.pairwise_packed(w.a, w.b, max_dist=k, dtype="uint8")
            np.testing.assert_array_equal(got, want, err_msg=f"{sched} k={k}")
            batch = gpu.PairsBatch(w.a, w.b)
            out = batch.run(batch.alloc("uint8"), max_dist=k)
            np.testing.assert_array_equal(out.get(), want, err_msg=f"{sched} k={k} resident")
    finally:
        gpu.set_schedule("auto")
