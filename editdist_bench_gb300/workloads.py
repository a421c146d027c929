"""Seeded synthetic workloads of the five benchmark shapes (numpy PCG64).

The reference measures on its own generator (bench/datagen.py:94-119:
a fixed number of edits per string, substitutions forced to change the
character).  These workloads follow the benchmark configuration instead:

* edits are i.i.d. per position with probability ``rate``; the kind is
  uniform over {substitute, insert-before, delete}; substituted and
  inserted symbols are drawn from the workload's symbol distribution and
  may equal the original symbol;
* data seed = 1000 + config number, scheduler-training seed = 2000 + config.

Every generator returns packed arrays ``(buf uint8, off int64[n+1])`` — the
layout of the reference's ``_edpy.pack`` (csrc/edpy.c:200-224) — so inputs
go to the engine without a Python string per item.
"""
from __future__ import annotations

import os
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass, field

import numpy as np

DNA = np.frombuffer(b"ACGT", dtype=np.uint8)
DNA_N = np.frombuffer(b"ACGTN", dtype=np.uint8)
DNA_N_P = np.array([0.2475, 0.2475, 0.2475, 0.2475, 0.01])


def _symbols(rng, n, alphabet, probs=None) -> np.ndarray:
    """n i.i.d. symbols of `alphabet`, uniform or with probabilities `probs`.
    Probabilities that are multiples of 1/D for a small D (the benchmark's
    {A,C,G,T: 0.2475, N: 0.01} is 99/400 and 4/400) are drawn as integers
    in [0, D) through a lookup table, which is exact and far faster than a
    weighted choice over hundreds of millions of draws."""
    if probs is None:
        return alphabet[rng.integers(0, len(alphabet), n, dtype=np.int64)]
    probs = np.asarray(probs, dtype=np.float64)
    for d in (100, 400, 1000, 10000):
        cnt = np.rint(probs * d)
        if np.allclose(cnt / d, probs, rtol=0, atol=1e-12) and cnt.sum() == d:
            table = np.repeat(alphabet, cnt.astype(np.int64))
            return table[rng.integers(0, d, n, dtype=np.int32)]
    return alphabet[rng.choice(len(alphabet), size=n, p=probs)]


_PAR_BYTES = 1 << 24          # sets larger than this are drawn in parallel pieces


def _pool():
    return ThreadPoolExecutor(max_workers=max(1, min(16, os.cpu_count() or 1)))


def random_strings(rng, lengths, alphabet=DNA, probs=None, parallel=True):
    """Packed i.i.d. strings with the given lengths. Large sets are drawn in
    pieces of 2^24 bytes on a thread pool, each piece from its own child
    generator of `rng` (numpy's generators release the GIL while filling)."""
    lengths = np.asarray(lengths, dtype=np.int64)
    off = np.zeros(len(lengths) + 1, dtype=np.int64)
    np.cumsum(lengths, out=off[1:])
    total = int(off[-1])
    if total <= _PAR_BYTES or not parallel:
        buf = _symbols(rng, total, alphabet, probs).astype(np.uint8)
        return _nonempty(buf), off
    cuts = list(range(0, total, _PAR_BYTES)) + [total]
    kids = rng.spawn(len(cuts) - 1)
    buf = np.empty(total, dtype=np.uint8)

    def piece(i):
        buf[cuts[i]:cuts[i + 1]] = _symbols(kids[i], cuts[i + 1] - cuts[i], alphabet, probs)
    with _pool() as ex:
        list(ex.map(piece, range(len(kids))))
    return buf, off


def _nonempty(buf):
    return buf if len(buf) else np.zeros(1, dtype=np.uint8)


def mutate(rng, packed, rates, alphabet=DNA, probs=None, chunk=1 << 16):
    """Apply i.i.d. per-position edits at per-string ``rates`` (scalar or
    array): a position is edited with probability rate; the edit is uniform
    over {substitute, insert-before, delete}; substitution and insertion
    draw a fresh symbol from the workload's distribution (it may equal the
    original). Strings are processed ``chunk`` at a time, each chunk with
    its own child generator of `rng` (on a thread pool when there are
    several); edit kinds and fresh symbols are drawn for edited positions
    only."""
    buf, off = packed
    n = len(off) - 1
    rates = np.broadcast_to(np.asarray(rates, dtype=np.float64), (n,))
    starts = list(range(0, n, chunk))
    kids = rng.spawn(len(starts))
    new_len = np.zeros(n, dtype=np.int64)

    def one(ci):
        r, i0 = kids[ci], starts[ci]
        i1 = min(n, i0 + chunk)
        p0, p1 = int(off[i0]), int(off[i1])
        lens = np.diff(off[i0:i1 + 1])
        orig = buf[p0:p1]
        pos = np.flatnonzero(r.random(p1 - p0) < np.repeat(rates[i0:i1], lens))   # edited positions
        op = r.integers(0, 3, len(pos), dtype=np.int8)                    # 0 sub, 1 insert-before, 2 delete
        fresh = _symbols(r, len(pos), alphabet, probs).astype(np.uint8)
        # every position emits its own symbol once (keep, substitute), twice
        # (insert-before: the fresh symbol, then the original) or not at all
        cnt = np.ones(p1 - p0, dtype=np.intp)
        cnt[pos[op == 1]] = 2
        cnt[pos[op == 2]] = 0
        out = np.repeat(orig, cnt)
        delta = (op == 1).astype(np.int64) - (op == 2)
        dest = pos + np.cumsum(delta) - delta                  # output index of each edited position
        out[dest[op == 0]] = fresh[op == 0]
        out[dest[op == 1]] = fresh[op == 1]
        sid = np.searchsorted(off[i0 + 1:i1 + 1] - p0, pos, side="right")   # string of each edit
        m = i1 - i0
        new_len[i0:i1] = lens + np.bincount(sid[op == 1], minlength=m) - np.bincount(sid[op == 2], minlength=m)
        return out

    if len(starts) > 1:
        with _pool() as ex:
            out_parts = list(ex.map(one, range(len(starts))))
    else:
        out_parts = [one(i) for i in range(len(starts))]
    noff = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(new_len, out=noff[1:])
    nbuf = np.concatenate(out_parts) if out_parts else np.zeros(0, dtype=np.uint8)
    return _nonempty(nbuf), noff


def take(packed, idx):
    """Packed subset (in the order of ``idx``)."""
    buf, off = packed
    idx = np.asarray(idx, dtype=np.int64)
    lengths = off[idx + 1] - off[idx]
    noff = np.zeros(len(idx) + 1, dtype=np.int64)
    np.cumsum(lengths, out=noff[1:])
    total = int(noff[-1])
    if total == 0:
        return np.zeros(1, dtype=np.uint8), noff
    src = np.repeat(off[idx] - noff[:-1], lengths) + np.arange(total, dtype=np.int64)
    return buf[src], noff


def concat(*packs):
    bufs, offs, base = [], [np.zeros(1, dtype=np.int64)], 0
    for buf, off in packs:
        nbytes = int(off[-1])
        bufs.append(buf[:nbytes])
        offs.append(off[1:] + base)
        base += nbytes
    buf = np.concatenate(bufs) if bufs else np.zeros(0, dtype=np.uint8)
    return _nonempty(buf), np.concatenate(offs)


def unpack(packed):
    buf, off = packed
    b = buf.tobytes()
    return [b[off[i]:off[i + 1]] for i in range(len(off) - 1)]


def cells(pa, pb) -> float:
    """Untrimmed DP cells sum(len a * len b) (bench/run_prior_art.py:182,245)."""
    return float(np.dot(np.diff(pa[1]).astype(np.float64), np.diff(pb[1]).astype(np.float64)))


def cross_cells(pq, pc) -> float:
    return float(np.diff(pq[1]).sum()) * float(np.diff(pc[1]).sum())


# ---------------------------------------------------------------- configs --
@dataclass
class PairsWork:
    name: str
    a: tuple
    b: tuple
    max_dist: int | None
    dtype: str
    meta: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return len(self.a[1]) - 1


@dataclass
class SearchWork:
    name: str
    q: tuple
    c: tuple
    max_dist: int | None
    dtype: str
    meta: dict = field(default_factory=dict)

    @property
    def nq(self) -> int:
        return len(self.q[1]) - 1

    @property
    def nc(self) -> int:
        return len(self.c[1]) - 1


def config1(n=1 << 20, seed=1001) -> PairsWork:
    """pairwise: a ~ U{ACGT}^32, b = a mutated at 5%; exact, int32."""
    rng = np.random.default_rng(seed)
    a = random_strings(rng, np.full(n, 32))
    b = mutate(rng, a, 0.05)
    return PairsWork("pairs-L32-dna-e0.05", a, b, None, "int32", {"n": n})


def config2(nq=4096, nc=65536, seed=1002, max_dist=None, dtype="int32") -> SearchWork:
    """cdist: 4096 queries x 65536 choices, length 64 over U{ACGT}; 1% of
    choices are copies of a random query mutated at 3%."""
    rng = np.random.default_rng(seed)
    q = random_strings(rng, np.full(nq, 64))
    n_plant = nc // 100
    plant_rows = rng.choice(nc, size=n_plant, replace=False)
    src = rng.integers(0, nq, n_plant)
    planted = mutate(rng, take(q, src), 0.03)
    rest_mask = np.ones(nc, dtype=bool)
    rest_mask[plant_rows] = False
    rest = random_strings(rng, np.full(nc - n_plant, 64))
    # interleave: planted rows at their positions, independent strings elsewhere
    order = np.empty(nc, dtype=np.int64)
    order[plant_rows] = np.arange(n_plant)
    order[rest_mask] = n_plant + np.arange(nc - n_plant)
    c = take(concat(planted, rest), order)
    return SearchWork("cdist-L64-dna", q, c, max_dist, dtype,
                      {"nq": nq, "nc": nc, "planted": n_plant})


def config3(n=1 << 22, seed=1003) -> PairsWork:
    """uneven pairs: |a| ~ U[8,256] over {ACGT: .2475, N: .01}; b = a mutated
    at a per-pair rate ~ U[0, 0.30]; max_dist 8, uint8."""
    rng = np.random.default_rng(seed)
    la = rng.integers(8, 257, n)
    a = random_strings(rng, la, DNA_N, DNA_N_P)
    rates = rng.uniform(0.0, 0.30, n)
    b = mutate(rng, a, rates, DNA_N, DNA_N_P)
    return PairsWork("pairs-uneven-L8-256-dnaN", a, b, 8, "uint8", {"n": n})


def config4(nq=1024, nc=1 << 20, seed=1004) -> SearchWork:
    """learned-ordered cdist: lengths ~ U[100,256] over U{ACGT}; 5% of the
    choices are mutants of a random query at a rate ~ U[0, 0.05];
    max_dist 4, uint8."""
    rng = np.random.default_rng(seed)
    q = random_strings(rng, rng.integers(100, 257, nq))
    n_plant = nc * 5 // 100
    plant_rows = rng.choice(nc, size=n_plant, replace=False)
    src = rng.integers(0, nq, n_plant)
    planted = mutate(rng, take(q, src), rng.uniform(0.0, 0.05, n_plant))
    rest = random_strings(rng, rng.integers(100, 257, nc - n_plant))
    rest_mask = np.ones(nc, dtype=bool)
    rest_mask[plant_rows] = False
    order = np.empty(nc, dtype=np.int64)
    order[plant_rows] = np.arange(n_plant)
    order[rest_mask] = n_plant + np.arange(nc - n_plant)
    c = take(concat(planted, rest), order)
    return SearchWork("cdist-L100-256-dna-k4", q, c, 4, "uint8",
                      {"nq": nq, "nc": nc, "planted": n_plant})


def config5(n_problems=256, seed=1005, scale=1.0):
    """mixed many-problem batch: query counts log-uniform in [1,512], choice
    counts log-uniform in [1024, 262144] (times ``scale``), lengths ~
    U[16,256] over U{ACGT}, max_dist ~ U{0..8}, dtype ~ U{int32,uint16,uint8}.
    The problems' shapes come from `seed` first; each problem's strings then
    come from its own child generator, on a thread pool."""
    rng = np.random.default_rng(seed)
    dts = ("int32", "uint16", "uint8")
    shapes = []
    for _ in range(n_problems):
        nq = int(np.exp(rng.uniform(np.log(1), np.log(512 + 1))))
        nq = max(1, min(512, nq))
        nc = int(np.exp(rng.uniform(np.log(1024), np.log(262144 + 1))))
        nc = max(1, min(262144, int(nc * scale)))
        shapes.append((nq, nc, int(rng.integers(0, 9)), dts[int(rng.integers(0, 3))]))
    kids = rng.spawn(n_problems)

    def one(i):
        nq, nc, k, dt = shapes[i]
        r = kids[i]
        q = random_strings(r, r.integers(16, 257, nq), parallel=False)
        c = random_strings(r, r.integers(16, 257, nc), parallel=False)
        return SearchWork(f"problem{i}", q, c, k, dt, {"nq": nq, "nc": nc})
    with _pool() as ex:
        return list(ex.map(one, range(n_problems)))
