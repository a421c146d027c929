#!/usr/bin/env python3
"""Benchmark of the GB300 Levenshtein engine — one JSON line on stdout.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--config 2] [--impl ours|reference]

Default workload (the reference's headline search shape): cdist of 4096
queries x 65536 choices, length 64 over uniform {A,C,G,T}, 1% planted
mutants; exact distances, int32 output. A step is one full pass of that
matrix. The metric is pairs/s (distances per second; GCUPS beside it).

* value:   kernel-only throughput — inputs resident in HBM, results left in
           HBM (the reference's "kernel-only" protocol, bench/baselines.py:
           150-160), CUDA events on the library's stream around each step,
           L2 flushed by a 256 MB memset between steps (outside the events).
* e2e:     the same metric through the C-ABI one-call entry point with host
           buffers: H2D of the packed inputs, kernels, D2H of the matrix.
* roofline: the dominant kernel's algorithmic integer operations per step
           (15 per 32-bit word-step) over its event-timed
           duration, against the integer-pipe peak measured on this GPU by
           libblg_probe.so; its HBM figure; and its issue-slot utilisation
           (warp instructions per pair from its ncu summary in profiles/,
           over SMs x 4 issue slots x the sampled SM clock).
* cpu_baseline: the oracle's C restatement of the reference's CPU core on a
           bounded sample, all host threads.
* matches: for a thresholded search, the same search in its matches-only
           form (sorted (query, choice, distance) records instead of the
           dense matrix), kernel-only and end to end; and (e2e_u4) the dense
           matrix end to end with 4-bit results, two per byte.
* runs:    the headline's max_dist=2 uint8 run, and each of the other four
           benchmark configurations (config1 .. config5 but the headline):
           kernel-only pairs/s, e2e, a CPU sample, the dominant kernel's
           roofline (HBM, integer pipe, issue slots) and, for the uneven
           pairs (3) and the thresholded search (4), every work order side
           by side (plain = the reference's natural order, auto, lensort,
           learned with its training time). --no-suite skips them.
* --impl reference: the reference's CPU path (here: the oracle port, since
           the reference's sources are not on the GPU host) on the same
           workload, all host threads; beside it ("reference_cuda") the
           reference's own CUDA kernels, compiled for sm_103a from its
           sources, timed kernel-only on this GPU where that cubin exists,
           and the same for the other four configurations
           ("reference_cuda_runs").

Under torchrun (N > 1) every rank runs its own replica of the workload on
its own GPU (weak scaling, no data-path collective); rank 0 reports the
aggregate over the max-over-ranks time.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from editdist_bench_gb300 import _build, _lib, gpu, workloads as W  # noqa: E402

H100_REF = {  # the reference's published kernel-only numbers (H100 SXM)
    1: (4.65e9, "H100 pairs kernel-only dna L32 5% 1M int32 (results/gpu-NVIDIA-H100-80GB-HBM3/prior_art_20261107-075217.csv:26)"),
    2: (6.1e9, "H100 search kernel-only dna L64 2000x2000 int32 (results/gpu-NVIDIA-H100-80GB-HBM3/prior_art_20261107-075006.csv:60)"),
}
L2_FLUSH_BYTES = 256 << 20
OPS_PER_WORD32_STEP = 15


# ------------------------------------------------------------------ ranks --
class Ranks:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist      # plumbing only: barrier + max over ranks
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo", rank=self.rank, world_size=self.world)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x: float) -> float:
        if not self.pg:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


# ----------------------------------------------------------------- clocks --
class Clocks:
    """nvidia-smi sampling during the timed region (SM MHz + throttle reasons)."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            t0 = time.time()                        # the sampler is running before the timed region opens
            while not self.rows and time.time() - t0 < 3.0 and self.proc.poll() is None:
                time.sleep(0.01)
            self.n_before = len(self.rows)
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self) -> dict:
        if self.proc:
            # a timed region shorter than the sampling period still gets the
            # first sample taken after it (the clocks of the just-ended load)
            t0 = time.time()
            while len(self.rows) <= getattr(self, "n_before", 0) and time.time() - t0 < 0.5:
                time.sleep(0.01)
            self.rows = self.rows[max(0, getattr(self, "n_before", 1) - 1):]
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows),
                "power_w_max": max((float(r[3]) for r in self.rows
                                    if r[3].replace(".", "").isdigit()), default=None)}


# ---------------------------------------------------------------- helpers --
def device_timer(ctx):
    lib = ctx.lib

    def start():
        ctx.check(lib.blg_timer_start(ctx.h))

    def stop() -> float:
        ms = ctypes.c_float()
        ctx.check(lib.blg_timer_stop(ctx.h, ctypes.byref(ms)))
        return float(ms.value)
    return start, stop


class Pinned:
    """Page-locked host copies (blg_host_alloc) of the e2e leg's inputs and
    outputs: the contract's host->device copies start from pinned memory."""

    def __init__(self, ctx):
        self.ctx = ctx
        self.ptrs = []

    def empty(self, shape, dtype):
        dtype = np.dtype(dtype)
        nbytes = max(1, int(np.prod(shape)) * dtype.itemsize)
        p = ctypes.c_void_p()
        self.ctx.check(self.ctx.lib.blg_host_alloc(self.ctx.h, ctypes.c_size_t(nbytes), ctypes.byref(p)))
        self.ptrs.append(p.value)
        raw = (ctypes.c_uint8 * nbytes).from_address(p.value)
        return np.frombuffer(raw, dtype=np.uint8)[:int(np.prod(shape)) * dtype.itemsize].view(dtype).reshape(shape)

    def copy(self, arr):
        out = self.empty(arr.shape, arr.dtype)
        out[...] = arr
        return out

    def packed(self, pk):
        return self.copy(pk[0]), self.copy(pk[1])

    def free(self):
        for p in self.ptrs:
            self.ctx.lib.blg_host_free(self.ctx.h, p)
        self.ptrs = []


def flush_l2(ctx, buf):
    ctx.check(ctx.lib.blg_memset(ctx.h, buf.ptr, 0x5a, ctypes.c_size_t(L2_FLUSH_BYTES)))


def int_peak(device: int) -> dict:
    lib = ctypes.CDLL(_build.build_probe())
    lib.blg_probe_int_peak.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                       ctypes.POINTER(ctypes.c_double)]
    a, b = ctypes.c_double(), ctypes.c_double()
    rc = lib.blg_probe_int_peak(device, 4096, ctypes.byref(a), ctypes.byref(b))
    if rc:
        return {"gops": None}
    return {"logic_gops": a.value / 1e9, "mixed_gops": b.value / 1e9,
            "gops": max(a.value, b.value) / 1e9}


def effective_cpus() -> int:
    """min(affinity, cgroup quota) — the rule of bench/sysload.py:19-41."""
    n = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
    try:
        q, period = open("/sys/fs/cgroup/cpu.max").read().split()[:2]
        if q != "max":
            n = min(n, max(1, int(int(q) / int(period))))
    except (OSError, ValueError):
        pass
    return max(1, n)


# -------------------------------------------------------------- workloads --
class SearchBench:
    kind = "cdist"

    def __init__(self, w: W.SearchWork, runs):
        self.w = w
        self.runs = runs                  # [(max_dist, dtype), ...]; runs[0] is the headline
        self.pairs = w.nq * w.nc
        self.cells = W.cross_cells(w.q, w.c)
        self.batch = gpu.SearchBatch(w.q, w.c)
        self.outs = [self.batch.alloc(dt) for _, dt in runs]
        self._host_out = {}

    def step(self, i=0):
        k, _ = self.runs[i]
        self.batch.run(self.outs[i], max_dist=k)

    def e2e_setup(self, pin):
        self._pq, self._pc = pin.packed(self.w.q), pin.packed(self.w.c)
        self._host_out = {i: pin.empty((self.w.nq, self.w.nc), dt) for i, (_, dt) in enumerate(self.runs)}

    def e2e_call(self, i=0):
        k, dt = self.runs[i]
        out = self._host_out[i]
        ctx = _lib.context()
        (bq, oq), (bc, oc) = self._pq, self._pc
        ctx.check(ctx.lib.blg_cdist(ctx.h, bq.ctypes.data, oq.ctypes.data, self.w.nq, bc.ctypes.data,
                                    oc.ctypes.data, self.w.nc, -1 if k is None else k,
                                    {"int32": 0, "uint16": 1, "uint8": 2}[dt], out.ctypes.data, None))
        return out

    def io_bytes(self, i=0):
        (bq, oq), (bc, oc) = self.w.q, self.w.c
        h2d = int(oq[-1]) + oq.nbytes + int(oc[-1]) + oc.nbytes
        return h2d, self.pairs * np.dtype(self.runs[i][1]).itemsize

    def alg_ops(self, i=0, exit_cols_sum=None):
        """15 x sum over pairs of ceil(m/32) x columns processed."""
        words = np.sum((np.diff(self.w.q[1]) + 31) // 32).astype(np.float64)
        if self.runs[i][0] is None:
            return OPS_PER_WORD32_STEP * words * float(np.diff(self.w.c[1]).sum())
        return None if exit_cols_sum is None else OPS_PER_WORD32_STEP * exit_cols_sum

    def alg_bytes(self, i=0):
        return self.pairs * np.dtype(self.runs[i][1]).itemsize + float(self.w.q[1][-1] + self.w.c[1][-1])

    def describe(self):
        return {"workload": f"{self.w.name} cdist {self.w.nq}x{self.w.nc}",
                "nq": self.w.nq, "nc": self.w.nc, "runs": [
                    {"max_dist": k, "dtype": dt} for k, dt in self.runs]}

    def cpu_sample(self, threads: int, budget_s: float):
        """Oracle on a bounded row sample; returns (pairs/s, sample text, rows, result)."""
        import oracle
        k, dt = self.runs[0]
        rows = max(1, min(self.w.nq, 8))
        while True:
            sub = W.take(self.w.q, np.arange(rows))
            t0 = time.perf_counter()
            res = oracle.cross(sub, self.w.c, k, threads=threads)
            dt_s = time.perf_counter() - t0
            if dt_s > budget_s / 4 or rows >= self.w.nq:
                break
            rows = min(self.w.nq, max(rows + 1, int(rows * budget_s / 4 / max(dt_s, 1e-3))))
        return rows * self.w.nc / dt_s, f"{rows} query rows x {self.w.nc} choices", rows, res

    def gate(self, rows, res) -> bool:
        got = self.outs[0].get()[:rows]
        return bool(np.array_equal(got, res.astype(got.dtype)))


class PairsBench:
    kind = "pairwise"

    def __init__(self, w: W.PairsWork):
        self.w = w
        self.runs = [(w.max_dist, w.dtype)]
        self.pairs = w.n
        self.cells = W.cells(w.a, w.b)
        self.batch = gpu.PairsBatch(w.a, w.b)
        self.outs = [self.batch.alloc(w.dtype)]
        self._host = None

    def step(self, i=0):
        self.batch.run(self.outs[0], max_dist=self.w.max_dist)

    def e2e_setup(self, pin):
        self._pa, self._pb = pin.packed(self.w.a), pin.packed(self.w.b)
        self._host = pin.empty((self.w.n,), self.w.dtype)

    def e2e_call(self, i=0):
        ctx = _lib.context()
        (ba, oa), (bb, ob) = self._pa, self._pb
        k = self.w.max_dist
        ctx.check(ctx.lib.blg_pairwise(ctx.h, ba.ctypes.data, oa.ctypes.data, bb.ctypes.data,
                                       ob.ctypes.data, self.w.n, -1 if k is None else k,
                                       {"int32": 0, "uint16": 1, "uint8": 2}[self.w.dtype],
                                       self._host.ctypes.data, None))
        return self._host

    def io_bytes(self, i=0):
        (ba, oa), (bb, ob) = self.w.a, self.w.b
        return int(oa[-1]) + oa.nbytes + int(ob[-1]) + ob.nbytes, self.w.n * np.dtype(self.w.dtype).itemsize

    def alg_ops(self, i=0, exit_cols_sum=None):
        return None if exit_cols_sum is None else OPS_PER_WORD32_STEP * exit_cols_sum

    def alg_bytes(self, i=0):
        (ba, oa), (bb, ob) = self.w.a, self.w.b
        return float(oa[-1] + ob[-1] + oa.nbytes + ob.nbytes + self.w.n * np.dtype(self.w.dtype).itemsize)

    def describe(self):
        return {"workload": f"{self.w.name} pairwise {self.w.n}", "n": self.w.n,
                "runs": [{"max_dist": self.w.max_dist, "dtype": self.w.dtype}]}

    def cpu_sample(self, threads: int, budget_s: float):
        import oracle
        n = min(self.w.n, 1 << 14)
        while True:
            sub_a = W.take(self.w.a, np.arange(n))
            sub_b = W.take(self.w.b, np.arange(n))
            t0 = time.perf_counter()
            res = oracle.pairs(sub_a, sub_b, self.w.max_dist, threads=threads)
            dt_s = time.perf_counter() - t0
            if dt_s > budget_s / 4 or n >= self.w.n:
                break
            n = min(self.w.n, max(n + 1, int(n * budget_s / 4 / max(dt_s, 1e-3))))
        return n / dt_s, f"first {n} pairs", n, res

    def gate(self, n, res) -> bool:
        got = self.outs[0].get()[:n]
        import oracle
        return bool(np.array_equal(got, oracle.saturate(res, self.w.dtype)))


class BatchBench:
    """The mixed many-problem batch: one step = one replay of the batch's graph."""
    kind = "batch"

    def __init__(self, probs):
        self.probs = probs
        self.runs = [("mixed", "mixed")]
        self.batch = gpu.ProblemBatch([(p.q, p.c, p.max_dist, p.dtype) for p in probs])
        self.pairs = self.batch.pairs
        self.cells = sum(W.cross_cells(p.q, p.c) for p in probs)
        self.outs = self.batch.outputs
        self.w = type("Batch", (), {"name": "cdist-batch-256-mixed"})()
        self._structs = None

    def step(self, i=0):
        self.batch.run()

    def e2e_setup(self, pin):
        self._pinned = [(pin.packed(p.q), pin.packed(p.c)) for p in self.probs]
        s = [_lib.Problem(q[0].ctypes.data, q[1].ctypes.data, p.nq, c[0].ctypes.data, c[1].ctypes.data,
                          p.nc, -1 if p.max_dist is None else p.max_dist,
                          {"int32": 0, "uint16": 1, "uint8": 2}[p.dtype], o.ptr)
             for p, o, (q, c) in zip(self.probs, self.outs, self._pinned)]
        self._structs = (_lib.Problem * len(s))(*s)

    def e2e_call(self, i=0):
        """Pinned host inputs -> one-call C-ABI (upload, graph, sync) into the device outputs."""
        ctx = _lib.context()
        ctx.check(ctx.lib.blg_cdist_batch(ctx.h, self._structs, len(self.probs)))

    def io_bytes(self, i=0):
        h2d = sum(int(p.q[1][-1]) + p.q[1].nbytes + int(p.c[1][-1]) + p.c[1].nbytes for p in self.probs)
        return h2d, 4          # results stay on the device (return_device); the status word comes back

    def alg_ops(self, i=0, exit_cols_sum=None):
        return None if exit_cols_sum is None else OPS_PER_WORD32_STEP * exit_cols_sum

    def alg_bytes(self, i=0):
        return float(sum(p.nq * p.nc * np.dtype(p.dtype).itemsize + p.q[1][-1] + p.c[1][-1] for p in self.probs))

    def describe(self):
        return {"workload": f"cdist batch of {len(self.probs)} problems", "problems": len(self.probs),
                "pairs": self.pairs, "runs": [{"max_dist": "mixed 0..8", "dtype": "mixed int32/uint16/uint8"}]}

    def cpu_sample(self, threads: int, budget_s: float):
        import oracle
        done, t0, res = 0, time.perf_counter(), None
        for p in self.probs:                       # smallest problems first, until the budget is spent
            rows = max(1, min(p.nq, 4))
            sub = W.take(p.q, np.arange(rows))
            oracle.cross(sub, p.c, p.max_dist, threads=threads)
            done += rows * p.nc
            if time.perf_counter() - t0 > budget_s / 4:
                break
        dt_s = time.perf_counter() - t0
        return done / dt_s, f"up to 4 query rows of each problem, {done} pairs", 0, res

    def gate(self, n, res) -> bool:
        import oracle
        p, o = self.probs[0], self.outs[0]
        return bool(np.array_equal(o.get(), oracle.saturate(oracle.cross(p.q, p.c, p.max_dist), p.dtype)))


def matches_leg(bench, ctx, pin, flush, args):
    """The same thresholded search in its matches-only form (records of the
    pairs with d <= max_dist, sorted): kernel-only through a resident
    search (blg_search_matches, records left in HBM, the count read back)
    and one-call from pinned host buffers (blg_cdist_matches)."""
    k = bench.runs[0][0]
    if k is None or bench.kind != "cdist":
        return None
    start, stop = device_timer(ctx)
    n = bench.batch.matches_into(bench.batch.match_buffer(1), k)
    buf = bench.batch.match_buffer(max(n, 1))
    for _ in range(3):
        bench.batch.matches_into(buf, k)
    t = []
    for _ in range(max(3, min(args.steps, 10))):
        flush_l2(ctx, flush)
        start()
        bench.batch.matches_into(buf, k)
        t.append(stop())
    ms = statistics.median(t)
    (bq, oq), (bc, oc) = bench._pq, bench._pc
    rec = pin.empty((max(n, 1),), gpu.MATCH_DTYPE)
    cnt = ctypes.c_int64()

    def call():
        ctx.check(ctx.lib.blg_cdist_matches(ctx.h, bq.ctypes.data, oq.ctypes.data, bench.w.nq, bc.ctypes.data,
                                            oc.ctypes.data, bench.w.nc, k, rec.ctypes.data, rec.shape[0],
                                            ctypes.byref(cnt)))
    for _ in range(3):
        call()
    e = []
    for _ in range(max(3, min(args.steps, 10))):
        t0 = time.perf_counter()
        call()
        e.append(time.perf_counter() - t0)
    e_s = statistics.median(e)
    assert cnt.value == n
    h2d, _ = bench.io_bytes(0)
    return {"matches": int(n), "record_bytes": gpu.MATCH_DTYPE.itemsize,
            "value": bench.pairs / (ms / 1e3), "unit": "pairs/s", "ms_per_step": ms,
            "e2e": {"value": bench.pairs / e_s, "unit": "pairs/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": int(n) * gpu.MATCH_DTYPE.itemsize + 8,
                    "path": "blg_cdist_matches, pinned host buffers, wall clock"},
            "path": ("blg_search_matches on the resident search: the survivor kernel's result list (no output, no "
                     "fill), sorted into records on the host and copied to HBM; CUDA events")}


def exit_columns(bench, sample_rows_or_n):
    """Oracle trace (columns processed under the reference's exit rule) on the
    CPU sample, scaled to the full workload — algorithmic ops for max_dist runs."""
    import oracle
    if bench.kind == "cdist":
        rows = sample_rows_or_n
        sub = W.take(bench.w.q, np.arange(rows))
        _, cols = oracle.cross_trace(sub, bench.w.c, bench.runs[0][0])
        words = ((np.diff(sub[1]) + 31) // 32).astype(np.float64)
        s = float((cols.astype(np.float64) * words[:, None]).sum())
        return s * bench.w.nq / rows
    if bench.kind == "batch":
        # up to 4 query rows of every problem, scaled by its query count
        total = 0.0
        for p in bench.probs:
            rows = min(p.nq, 4)
            if rows == 0 or p.nc == 0:
                continue
            sub = W.take(p.q, np.arange(rows))
            _, cols = oracle.cross_trace(sub, p.c, p.max_dist)
            words = ((np.diff(sub[1]) + 31) // 32).astype(np.float64)
            total += float((cols.astype(np.float64) * words[:, None]).sum()) * p.nq / rows
        return total
    n = sample_rows_or_n
    sa, sb = W.take(bench.w.a, np.arange(n)), W.take(bench.w.b, np.arange(n))
    _, m, _, cols = oracle.pairs_trace(sa, sb, bench.w.max_dist)
    s = float((((m.astype(np.float64) + 31) // 32) * cols).sum())
    return s * bench.w.n / n


def make_bench(cfg: int, args=None):
    """Benchmark configuration `cfg`; --nq/--nc/--n shrink it (profiling runs)."""
    nq = getattr(args, "nq", None)
    nc = getattr(args, "nc", None)
    n = getattr(args, "n", None)
    if cfg == 1:
        return PairsBench(W.config1(n=n or (1 << 20)))
    if cfg == 2:
        return SearchBench(W.config2(nq=nq or 4096, nc=nc or 65536), [(None, "int32"), (2, "uint8")])
    if cfg == 3:
        return PairsBench(W.config3(n=n or (1 << 22)))
    if cfg == 4:
        return SearchBench(W.config4(nq=nq or 1024, nc=nc or (1 << 20)), [(4, "uint8")])
    if cfg == 5:
        return BatchBench(W.config5(scale=getattr(args, "scale", 1.0) or 1.0))
    raise SystemExit(f"unknown config {cfg}")


def hbm_peak() -> tuple:
    """Measured copy bandwidth of this GPU pool (MEASURED_PEAKS.json, written
    beside this file by the environment), else the fallback figure."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs)"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback 6.8 TB/s"


def read_profile(kernel: str, workload: str) -> dict:
    """Machine-readable ``key=value`` lines of the committed ncu summary of a
    kernel launch label on a workload (profiles/<label>_<workload>.txt):
    traffic_bytes_per_launch (DRAM bytes of a full launch), inst_per_unit
    (warp instructions per pair, all launches of the label in one step),
    time_share (the counted kernel's share of the label's time, when the
    label is a graph of several kernels), alu_pipe / issue_active (ncu's
    pipe and issue utilisation)."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_{workload}.txt")
    out = {"path": os.path.relpath(path, ROOT)}
    try:
        for line in open(path):
            if "=" in line and not line.startswith((" ", "#")):
                k, v = line.strip().split("=", 1)
                try:
                    out[k] = float(v)
                except ValueError:
                    out[k] = v
    except OSError:
        return {}
    return out


def device_info(device: int) -> dict:
    lib = ctypes.CDLL(_build.build_probe())
    sms, khz = ctypes.c_int(), ctypes.c_int()
    if lib.blg_probe_device_info(device, ctypes.byref(sms), ctypes.byref(khz)):
        return {}
    return {"sms": sms.value, "max_mhz": khz.value / 1e3}


def train_scheduler(ctx, cfg: int, args) -> dict:
    """Train the work-order network on up to 2^20 logged rows of the same
    workload shape drawn with a different seed (2000 + config), outside the
    timed region: pairs for configs 1 and 3; for config 4 the survivors of 64
    queries against 2^20 choices (the thresholded search's own rows)."""
    if cfg == 4:
        t0 = time.perf_counter()
        w = W.config4(nq=64, nc=1 << 20, seed=2004)
        batch = gpu.SearchBatch(w.q, w.c)
        t1 = time.perf_counter()
        loss = ctypes.c_float()
        ctx.check(ctx.lib.blg_sched_train_search(ctx.h, batch.h, w.max_dist, args.epochs, ctypes.c_float(args.lr),
                                                 1 << 20, ctypes.byref(loss)))
        t2 = time.perf_counter()
        return {"trained": True, "rows_max": 1 << 20, "seed": 2004, "rows_from": "64 queries x 2^20 choices",
                "epochs": args.epochs, "lr": args.lr, "final_mse": loss.value, "train_s": t2 - t1,
                "data_s": t1 - t0}
    gen = {1: W.config1, 3: W.config3}.get(cfg)
    if gen is None:
        return {"trained": False, "why": "the learned order applies to pairwise and thresholded-search workloads"}
    t0 = time.perf_counter()
    w = gen(n=1 << 20, seed=2000 + cfg)
    batch = gpu.PairsBatch(w.a, w.b)
    t1 = time.perf_counter()
    loss = ctypes.c_float()
    k = -1 if w.max_dist is None else w.max_dist
    ctx.check(ctx.lib.blg_sched_train(ctx.h, batch.h, k, args.epochs, ctypes.c_float(args.lr), 1 << 20,
                                      ctypes.byref(loss)))
    t2 = time.perf_counter()
    return {"trained": True, "rows_max": 1 << 20, "seed": 2000 + cfg, "epochs": args.epochs,
            "lr": args.lr, "final_mse": loss.value, "train_s": t2 - t1, "data_s": t1 - t0}


def timed_steps(ctx, flush, fn, steps):
    """CUDA-event times (ms) of `steps` calls of fn, L2 flushed before each."""
    start, stop = device_timer(ctx)
    times = []
    for _ in range(steps):
        flush_l2(ctx, flush)
        start()
        fn()
        times.append(stop())
    return times


def kernel_stats(ctx, flush, fn, reps=3):
    """Per-launch-label event timing of `reps` steps: ({label: {launches,
    total_ms}}, the label with the largest total)."""
    ctx.check(ctx.lib.blg_profile_enable(ctx.h, 1))
    for _ in range(reps):
        flush_l2(ctx, flush)
        fn()
    buf = ctypes.create_string_buffer(8192)
    ctx.check(ctx.lib.blg_profile_report(ctx.h, buf, 8192))
    ctx.check(ctx.lib.blg_profile_enable(ctx.h, 0))
    kstats = {}
    for line in buf.value.decode().splitlines():
        name, cnt, ms = line.split()
        kstats[name] = {"launches": int(cnt) / reps, "ms_per_step": float(ms) / reps}
    top = max(kstats, key=lambda n: kstats[n]["ms_per_step"]) if kstats else None
    return kstats, top


def e2e_leg(bench, pin, steps, warmup, i=0) -> dict:
    """The same metric through the one-call C-ABI from pinned host buffers:
    wall clock of whole calls (copies in, kernels, copies out)."""
    for _ in range(max(warmup, 3)):              # the first calls on fresh pinned pages run slow
        bench.e2e_call(i)
    t = []
    for _ in range(max(3, steps)):
        t0 = time.perf_counter()
        bench.e2e_call(i)
        t.append(time.perf_counter() - t0)
    s = statistics.median(t)
    h2d, d2h = bench.io_bytes(i)
    return {"value": bench.pairs / s, "unit": "pairs/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
            "ms_per_call": s * 1e3,
            "path": "one-call C-ABI (blg_pairwise / blg_cdist / blg_cdist_batch), pinned host buffers, wall clock"}


def u4_leg(bench, pin, steps: int, warmup: int) -> dict | None:
    """A thresholded search with max_dist <= 14 in its 4-bit form (BLG_UINT4:
    two results per byte, exact below 15): the one-call C-ABI from pinned
    host buffers, the packed matrix copied back (half of uint8's bytes)."""
    k = bench.runs[0][0]
    if bench.kind != "cdist" or k is None or k > 14:
        return None
    ctx = _lib.context()
    (bq, oq), (bc, oc) = bench._pq, bench._pc
    nbytes = (bench.w.nq * bench.w.nc + 1) // 2
    out = pin.empty((nbytes,), np.uint8)

    def call():
        ctx.check(ctx.lib.blg_cdist(ctx.h, bq.ctypes.data, oq.ctypes.data, bench.w.nq, bc.ctypes.data,
                                    oc.ctypes.data, bench.w.nc, k, _lib.UINT4, out.ctypes.data, None))
    for _ in range(max(warmup, 3)):
        call()
    t = []
    for _ in range(max(3, steps)):
        t0 = time.perf_counter()
        call()
        t.append(time.perf_counter() - t0)
    s = statistics.median(t)
    h2d, _ = bench.io_bytes(0)
    return {"value": bench.pairs / s, "unit": "pairs/s", "ms_per_call": s * 1e3, "h2d_bytes_per_step": h2d,
            "d2h_bytes_per_step": nbytes,
            "path": "blg_cdist with 4-bit results (two per byte), pinned host buffers, wall clock"}


def list_leg(bench, calls: int = 3) -> dict | None:
    """The drop-in call on Python lists of bytes, as a bitlev user makes it:
    gpu.pairwise(a, b) / gpu.cdist(q, c) with packing (the native packer into
    page-locked staging), the copies, the kernels and the result returned as
    a new numpy array, all inside the wall-clock time. The lists are built
    outside it."""
    from editdist_bench_gb300 import _common
    if bench.kind == "pairwise":
        a, b = W.unpack(bench.w.a), W.unpack(bench.w.b)
        k, dt = bench.runs[0]
        call = lambda: gpu.pairwise(a, b, max_dist=k, dtype=dt)  # noqa: E731
    elif bench.kind == "cdist":
        a, b = W.unpack(bench.w.q), W.unpack(bench.w.c)
        k, dt = bench.runs[0]
        call = lambda: gpu.cdist(a, b, max_dist=k, dtype=dt)  # noqa: E731
    else:
        return None
    call()
    t = []
    for _ in range(max(2, calls)):
        t0 = time.perf_counter()
        r = call()
        t.append(time.perf_counter() - t0)
        del r
    s = statistics.median(t)
    return {"value": bench.pairs / s, "unit": "pairs/s", "ms_per_call": s * 1e3, "calls": len(t),
            "packer": "native (csrc/blg_pack.c)" if _common._blgpack is not None else "python",
            "path": "gpu.pairwise / gpu.cdist on Python lists of bytes: packing into pinned staging, copies, "
                    "kernels, result into a new numpy array; wall clock"}


def roofline_block(bench, kstats, top, peak, exit_sum, dev, clock_mhz) -> dict:
    """The dominant launch label's roofline: algorithmic bytes and integer
    ops per step over its event time (HBM and integer-pipe fractions, the
    binding one first), plus its issue-slot utilisation from the warp
    instructions per pair its ncu summary records."""
    ms = kstats[top]["ms_per_step"]
    ops = bench.alg_ops(0, exit_sum)
    hpeak, hsrc = hbm_peak()
    hbm = {"achieved": bench.alg_bytes(0) / (ms / 1e3) / 1e9, "peak": hpeak, "unit": "GB/s",
           "peak_source": hsrc, "alg_bytes_per_step": bench.alg_bytes(0)}
    hbm["frac"] = hbm["achieved"] / hpeak
    ipart = {"peak": peak.get("gops"), "unit": "Gop/s",
             "peak_source": "measured: libblg_probe LOP3/IADD3 stream on this GPU", "peak_detail": peak}
    if ops is not None and peak.get("gops"):
        ipart["alg_ops_per_step"] = ops
        ipart["achieved"] = ops / (ms / 1e3) / 1e9
        ipart["frac"] = ipart["achieved"] / peak["gops"]
    prof = read_profile(top, bench.w.name)
    issue = None
    if prof.get("inst_per_unit") and dev.get("sms"):
        mhz = clock_mhz or dev["max_mhz"]
        share = prof.get("time_share", 1.0)   # the counted kernel's share of a label that spans several kernels
        slots = dev["sms"] * 4 * mhz * 1e6 * ms * share / 1e3
        inst = prof["inst_per_unit"] * bench.pairs
        issue = {"frac": inst / slots, "inst_per_unit": prof["inst_per_unit"], "unit": "warp instructions per pair",
                 "clock_mhz": mhz, "alu_pipe_ncu": prof.get("alu_pipe"), "issue_active_ncu": prof.get("issue_active"),
                 "time_share": share, "source": prof["path"],
                 "how": "inst_per_unit x pairs per step / (event ms x time_share x SMs x 4 issue slots per clock "
                        "x SM clock)"}
    # short exact pairs (config 1) are bound by moving their bytes; the rest by the integer pipe
    primary = hbm if (bench.kind == "pairwise" and bench.runs[0][0] is None) else ipart
    traffic = prof.get("traffic_bytes_per_launch")
    launches = kstats[top]["launches"]
    return {"kernel": top, "bound": "hbm" if primary is hbm else "int", "achieved": primary.get("achieved"),
            "peak": primary.get("peak"), "unit": primary["unit"], "frac": primary.get("frac"),
            "traffic": traffic, "ms_per_launch": ms / launches, "launches_per_step": launches,
            "int": ipart, "hbm": hbm, "issue": issue}


def cpu_leg(bench, budget_s: float) -> tuple:
    """The oracle on a bounded sample (all host threads, then one thread):
    the cpu_baseline object, and the exit-column total of the reference's
    rule scaled to the workload (the algorithmic ops of max_dist runs)."""
    threads = effective_cpus()
    v, sample, n_s, res = bench.cpu_sample(threads, budget_s)
    v1, sample1, _, _ = bench.cpu_sample(1, budget_s / 3)
    cpu = {"value": v, "unit": "pairs/s", "cores": threads, "kind": "port", "sample": sample,
           "single_thread": {"value": v1, "sample": sample1}, "gate": bench.gate(n_s, res)}
    exit_sum = None
    if bench.kind in ("pairwise", "batch") or bench.runs[0][0] is not None:
        exit_sum = exit_columns(bench, n_s)
    return cpu, exit_sum


SUITE_SCHEDULES = {3: ["plain", "auto", "lensort", "learned"], 4: ["plain", "auto", "lensort", "learned"]}


def suite_config(cfg, ctx, flush, pin, args, peak, dev, clock_mhz) -> dict:
    """One benchmark configuration besides the headline: kernel-only pairs/s
    under each work order it has, e2e, CPU sample, roofline."""
    t0 = time.perf_counter()
    bench = make_bench(cfg)
    gen_s = time.perf_counter() - t0
    steps = max(3, min(args.steps, 10))
    scheds = SUITE_SCHEDULES.get(cfg, ["auto"])
    res = {"workload": bench.describe()["workload"], "config": cfg, "data_gen_s": gen_s, "steps": steps,
           "warmup": args.warmup}
    sched_out = {}
    kstats = top = None
    try:
        for sch in scheds:
            gpu.set_schedule(sch)
            entry = {}
            if sch == "learned":
                entry["training"] = train_scheduler(ctx, cfg, args)
            for _ in range(args.warmup):
                bench.step(0)
            gpu.synchronize()
            ms = statistics.median(timed_steps(ctx, flush, lambda: bench.step(0), steps))
            entry.update({"value": bench.pairs / (ms / 1e3), "ms_per_step": ms,
                          "gcups": bench.cells / (ms / 1e3) / 1e9})
            sched_out[sch] = entry
            if sch == "auto":
                kstats, top = kernel_stats(ctx, flush, lambda: bench.step(0))
    finally:
        gpu.set_schedule("auto")
    a = sched_out["auto"]
    res.update({"value": a["value"], "unit": "pairs/s", "ms_per_step": a["ms_per_step"], "gcups": a["gcups"],
                "schedule": "auto", "kernels": kstats})
    if len(scheds) > 1:
        res["schedules"] = sched_out
        res["speedup_vs_plain"] = {s: sched_out["plain"]["ms_per_step"] / v["ms_per_step"]
                                   for s, v in sched_out.items() if s != "plain"}
    bench.e2e_setup(pin)
    res["e2e"] = e2e_leg(bench, pin, steps, args.warmup)
    if cfg in (1, 4):
        res["e2e_list"] = list_leg(bench)
    m = matches_leg(bench, ctx, pin, flush, args)
    if m:
        res["matches"] = m
    u4 = u4_leg(bench, pin, steps, args.warmup)
    if u4:
        res["e2e_u4"] = u4
    cpu, exit_sum = (None, None) if args.no_cpu_baseline else cpu_leg(bench, args.suite_cpu_budget)
    res["cpu_baseline"] = cpu
    if top:
        res["roofline"] = roofline_block(bench, kstats, top, peak, exit_sum, dev, clock_mhz)
    return res


# ------------------------------------------------------------------ arms --
def run_ours(args, ranks: Ranks):
    ctx = _lib.context()
    tune = None
    if not args.no_autotune:                     # launch shapes for this GPU, outside the timed region
        t0 = time.perf_counter()
        tune = gpu.autotune(os.path.join(tempfile.gettempdir(), f"blg_tune_{ranks.local}.txt"))
        tune["seconds"] = time.perf_counter() - t0
    gpu.set_schedule(args.schedule)
    bench = make_bench(args.config, args)
    p = ctypes.c_void_p()
    ctx.check(ctx.lib.blg_malloc(ctx.h, L2_FLUSH_BYTES, ctypes.byref(p)))
    flush = gpu.DeviceArray(p.value, (L2_FLUSH_BYTES,), np.uint8, ctx)

    sched_info = None
    if args.schedule == "learned":
        sched_info = train_scheduler(ctx, args.config, args)
    for i in range(len(bench.runs)):          # warm-up every run variant
        for _ in range(args.warmup):
            bench.step(i)
    gpu.synchronize()

    clocks = Clocks(ranks.local)
    clocks.start()
    for _ in range(20):                       # let the sampler start; keep the GPU busy meanwhile
        bench.step(0)
    gpu.synchronize()
    ranks.barrier()
    launches0 = ctx.lib.blg_launch_count(ctx.h)
    wall0 = time.perf_counter()
    times = timed_steps(ctx, flush, lambda: bench.step(0), args.steps)
    wall = time.perf_counter() - wall0
    launches = ctx.lib.blg_launch_count(ctx.h) - launches0
    gpu.synchronize()
    clk = clocks.stop()
    ranks.barrier()
    total_ms = ranks.max(sum(times))
    ms_per_step = total_ms / args.steps
    value = bench.pairs * ranks.world / (ms_per_step / 1e3)

    extra_runs = {}
    for i in range(1, len(bench.runs)):
        ms = statistics.median(timed_steps(ctx, flush, lambda: bench.step(i), max(3, args.steps // 2)))
        k, dt = bench.runs[i]
        extra_runs[f"max_dist={k},{dt}"] = {"pairs_per_s": bench.pairs / (ms / 1e3), "ms_per_step": ms,
                                            "gcups": bench.cells / (ms / 1e3) / 1e9}

    # per-kernel event timing for the roofline (a separate, profiled pass)
    kstats, top = kernel_stats(ctx, flush, lambda: bench.step(0))

    # e2e through the C-ABI with pinned host buffers
    pin = Pinned(ctx)
    e2e = matches = e2e_list = None
    if not args.kernel_only:
        bench.e2e_setup(pin)
        e2e = e2e_leg(bench, pin, min(args.steps, 10), args.warmup)
        e2e["value"] = bench.pairs * ranks.world / (ranks.max(bench.pairs / e2e["value"]))
        matches = matches_leg(bench, ctx, pin, flush, args)
        e2e_list = list_leg(bench) if ranks.world == 1 and not args.no_suite else None

    result = {
        "metric": "pairs/s", "value": value, "unit": "pairs/s", "n_gpus": ranks.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u64", "data": "synthetic (seeded numpy generator, workload shapes of the benchmark configuration)",
        "config": dict(bench.describe(), l2="flushed between steps (256 MB memset outside the timed events)",
                       parallelism="replicas" if ranks.world > 1 else "single GPU", schedule=args.schedule),
        "gcups": bench.cells * ranks.world / (ms_per_step / 1e3) / 1e9,
        "e2e": e2e,
        "gpu_launches": int(launches), "wall_s_timed_region": wall, "scheduler": sched_info, "tuning": tune,
        "clocks": clk, "runs": extra_runs, "kernels": kstats,
    }
    if matches:
        result["matches"] = matches
    if e2e_list:
        result["e2e_list"] = e2e_list
    if args.config in H100_REF:
        ref, src = H100_REF[args.config]
        result["vs_baseline"] = value / ref
        result["vs_baseline_ref"] = src

    if ranks.rank == 0:
        peak = int_peak(ranks.local)
        dev = device_info(ranks.local)
        exit_sum = None
        cpu = None
        if not args.no_cpu_baseline:
            cpu, exit_sum = cpu_leg(bench, args.cpu_budget)
        result["cpu_baseline"] = cpu
        if top:
            result["roofline"] = roofline_block(bench, kstats, top, peak, exit_sum, dev, clk.get("sm_mhz"))
        # the other benchmark configurations (rank 0 of a single-GPU run):
        # kernel-only, e2e, work orders, roofline each; results identical to
        # the oracle's by the parity tests
        if not args.no_suite and ranks.world == 1:
            del bench
            suite_t0 = time.perf_counter()
            for cfg in (1, 2, 3, 4, 5):
                if cfg == args.config:
                    continue
                result["runs"][f"config{cfg}"] = suite_config(cfg, ctx, flush, pin, args, peak, dev,
                                                              clk.get("sm_mhz"))
            result["suite_s"] = time.perf_counter() - suite_t0
        pin.free()
        print(json.dumps(result), flush=True)
    else:
        pin.free()


def reference_cuda_leg(w, steps: int, warmup: int) -> dict:
    """The reference's own CUDA kernels (csrc/gpu_kernels.cu compiled for
    sm_103a from its sources, launched with bitlev/gpu.py's geometry by
    oracle/ref_cuda.py) on the same workload, kernel-only, inputs resident."""
    from oracle import ref_cuda as RC
    if not RC.available():
        return {"unavailable": "the reference's CUDA kernels were not compiled (its sources are read where they lie, "
                               "so the cubin is built only where the reference checkout exists)"}
    r = RC.RefCuda(int(os.environ.get("BLG_DEVICE", "0")))
    try:
        probs = w if isinstance(w, list) else [w]
        runs, pairs = [], 0
        for p in probs:
            k = -1 if p.max_dist is None else int(p.max_dist)
            out8 = p.dtype == "uint8"
            item = 1 if out8 else 4                # uint16 is an int32 launch plus a conversion in bitlev
            if isinstance(p, W.SearchWork):
                st = r.cross_setup(p.q, p.c)
                out = r._keep(r.d.alloc(p.nq * p.nc * item))
                runs.append((r.cross_run, st, out, k, out8))
                pairs += p.nq * p.nc
            else:
                st = r.pairs_setup(p.a, p.b)
                out = r._keep(r.d.alloc(p.n * item))
                runs.append((r.pairs_run, st, out, k, out8))
                pairs += p.n

        def call():
            for fn, st, out, k, out8 in runs:
                fn(st, out, k, out8)
        t = r.time_calls(call, steps, warmup)
        ms = float(np.mean(t))
        return {"value": pairs / (ms / 1e3), "unit": "pairs/s", "ms_per_step": ms, "steps": steps,
                "kind": "reference kernels (csrc/gpu_kernels.cu) compiled for sm_103a, bitlev/gpu.py launch "
                        "geometry, CUDA events, inputs resident, L2 flushed between steps"}
    finally:
        r.close()


def run_reference(args, ranks: Ranks):
    """The reference's CPU path on the host cores (oracle port: the reference's
    sources are not present on the GPU host), same workload and metric; beside
    it, the reference's own CUDA kernels on this GPU where they were compiled."""
    if ranks.rank != 0:
        return
    import oracle
    cfg = args.config
    w = {1: W.config1, 2: W.config2, 3: W.config3, 4: W.config4, 5: W.config5}[cfg]()
    threads = effective_cpus()
    if isinstance(w, list):                        # the many-problem batch: up to 4 rows of each problem
        probs = w
        per = sum(min(p.nq, 4) * p.nc for p in probs)
        cells = sum(W.cross_cells(W.take(p.q, np.arange(min(p.nq, 4))), p.c) for p in probs)
        fn = lambda: [oracle.cross(W.take(p.q, np.arange(min(p.nq, 4))), p.c, p.max_dist,  # noqa: E731
                                   threads=threads) for p in probs]
        sample = f"up to 4 query rows of each of the {len(probs)} problems ({per} pairs) per step"
        workload = f"cdist batch of {len(probs)} problems"
    elif isinstance(w, W.SearchWork):
        k = w.max_dist
        rows = max(1, min(w.nq, 16 * threads))
        sub = W.take(w.q, np.arange(rows))
        fn = lambda: oracle.cross(sub, w.c, k, threads=threads)  # noqa: E731
        per = rows * w.nc
        cells = W.cross_cells(sub, w.c)
        sample = f"{rows} query rows x {w.nc} choices per step"
        workload = f"{w.name} cdist {w.nq}x{w.nc}"
    else:
        n = min(w.n, 1 << 18)
        sa, sb = W.take(w.a, np.arange(n)), W.take(w.b, np.arange(n))
        fn = lambda: oracle.pairs(sa, sb, w.max_dist, threads=threads)  # noqa: E731
        per = n
        cells = W.cells(sa, sb)
        sample = f"first {n} pairs per step"
        workload = f"{w.name} pairwise {w.n}"
    for _ in range(args.warmup):
        fn()
    t = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        fn()
        t.append(time.perf_counter() - t0)
    s = sum(t) / len(t)
    value = per / s
    try:
        ref_cuda = reference_cuda_leg(w, args.steps, max(args.warmup, 3))
    except Exception as e:                         # reported, never fatal to the CPU arm
        ref_cuda = {"unavailable": f"{type(e).__name__}: {e}"}
    # the reference's CUDA kernels on the other benchmark configurations too
    # (kernel-only, same GPU), beside the per-configuration lines of our arm
    ref_runs = {}
    if not args.no_suite and ranks.world == 1 and "unavailable" not in ref_cuda:
        del w
        for c2 in (1, 2, 3, 4, 5):
            if c2 == cfg:
                continue
            try:
                w2 = {1: W.config1, 2: W.config2, 3: W.config3, 4: W.config4, 5: W.config5}[c2]()
                ref_runs[f"config{c2}"] = reference_cuda_leg(w2, max(3, min(args.steps, 5)), 2)
                del w2
            except Exception as e:
                ref_runs[f"config{c2}"] = {"unavailable": f"{type(e).__name__}: {e}"}
    print(json.dumps({
        "impl": "reference", "metric": "pairs/s", "value": value, "unit": "pairs/s", "n_gpus": ranks.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": s * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u64", "data": "synthetic",
        "config": {"workload": workload, "sample": sample},
        "gcups": cells / s / 1e9,
        "cpu_baseline": {"value": value, "unit": "pairs/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "reference_cuda": ref_cuda,
        "reference_cuda_runs": ref_runs,
    }), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--config", type=int, default=2)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-budget", type=float, default=12.0, help="seconds of oracle work per leg")
    ap.add_argument("--suite-cpu-budget", type=float, default=3.0,
                    help="seconds of oracle work per leg for the other configurations")
    ap.add_argument("--kernel-only", action="store_true",
                    help="skip the end-to-end, matches and list legs (profiling runs)")
    ap.add_argument("--no-suite", action="store_true",
                    help="report the headline configuration only (not the other four under runs)")
    ap.add_argument("--nq", type=int, default=None, help="override the query count (profiling)")
    ap.add_argument("--nc", type=int, default=None, help="override the choice count (profiling)")
    ap.add_argument("--n", type=int, default=None, help="override the pair count (profiling)")
    ap.add_argument("--scale", type=float, default=None, help="shrink the batch's choice counts (config 5)")
    ap.add_argument("--schedule", default="auto", choices=["auto", "plain", "learned", "lensort"],
                    help="work order of max_dist runs (results are identical)")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch shapes")
    ap.add_argument("--epochs", type=int, default=10, help="scheduler training epochs (learned)")
    ap.add_argument("--lr", type=float, default=0.02, help="scheduler learning rate (learned)")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    ranks = Ranks()
    if ranks.world > 1:
        os.environ["BLG_DEVICE"] = str(ranks.local)
    try:
        if args.impl == "reference":
            run_reference(args, ranks)
        else:
            run_ours(args, ranks)
    finally:
        ranks.close()


if __name__ == "__main__":
    main()
