"""GPU parity: every result of the CUDA path (through the C-ABI, via the
ctypes drop-in module) must equal the reference's answers bit for bit —
the committed golden fixtures generated from the reference, and the oracle
on fresh seeded data. Mirrors the reference's GPU test strategy
(tests/test_cuda_gpu.py, tests/test_lib_gpu.py) without its CPU fallback."""
import random

import numpy as np
import pytest

import oracle
from editdist_bench_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _enc(s):
    return s.encode("latin-1")


def test_known_answers(gpu, known):
    A = [_enc(c["a"]) for c in known["exact"]]
    B = [_enc(c["b"]) for c in known["exact"]]
    want = [c["d"] for c in known["exact"]]
    assert gpu.pairwise(A, B).tolist() == want
    assert gpu.pairwise(B, A).tolist() == want
    for i in range(len(A)):
        assert gpu.cdist([A[i]], [B[i]])[0, 0] == want[i]
    for c in known["thresholded"]:
        a, b = _enc(c["a"]), _enc(c["b"])
        assert gpu.pairwise([a], [b], max_dist=c["k"])[0] == c["d"], c
        assert gpu.cdist([a], [b], max_dist=c["k"])[0, 0] == c["d"], c


def test_saturation(gpu, known):
    s = known["saturation"]
    for dt in ("int32", "uint8", "uint16"):
        got = gpu.cdist(s["Q"], s["C"], dtype=dt)
        assert got.dtype == np.dtype(dt) and got.tolist() == s[dt]
    assert gpu.pairwise(["x" * 300], [""], dtype=np.uint8)[0] == s["pair_x300_empty_uint8"]


def test_random_suite(gpu, rsuite):
    pa = (rsuite["a_buf"], rsuite["a_off"])
    pb = (rsuite["b_buf"], rsuite["b_off"])
    pq = (rsuite["q_buf"], rsuite["q_off"])
    pc = (rsuite["c_buf"], rsuite["c_off"])
    for key, want in rsuite.items():
        if not key.startswith(("pairs_", "cross_")):
            continue
        kind, kk, dt = key.split("_")
        k = None if kk == "knone" else int(kk[1:])
        if kind == "pairs":
            got = gpu.pairwise_packed(pa, pb, max_dist=k, dtype=dt)
        else:
            got = gpu.cdist_packed(pq, pc, max_dist=k, dtype=dt)
        assert got.dtype == want.dtype
        np.testing.assert_array_equal(got, want, err_msg=key)


def test_config_subsamples(gpu, csuite):
    for tag, k, dt in (("c1", None, "int32"), ("c3", 8, "uint8")):
        pa = (csuite[f"{tag}_a_buf"], csuite[f"{tag}_a_off"])
        pb = (csuite[f"{tag}_b_buf"], csuite[f"{tag}_b_off"])
        np.testing.assert_array_equal(gpu.pairwise_packed(pa, pb, k, dt), csuite[f"{tag}_out"])
    for tag, cases in (("c2", ((None, "int32"), (2, "uint8"))), ("c4", ((4, "uint8"),))):
        pq = (csuite[f"{tag}_q_buf"], csuite[f"{tag}_q_off"])
        pc = (csuite[f"{tag}_c_buf"], csuite[f"{tag}_c_off"])
        for k, dt in cases:
            want = csuite[f"{tag}_k{'none' if k is None else k}_{dt}"]
            np.testing.assert_array_equal(gpu.cdist_packed(pq, pc, k, dt), want)
    i = 0
    while f"c5_{i}_out" in csuite:
        pq = (csuite[f"c5_{i}_q_buf"], csuite[f"c5_{i}_q_off"])
        pc = (csuite[f"c5_{i}_c_buf"], csuite[f"c5_{i}_c_off"])
        k, dt = int(csuite[f"c5_{i}_k"][0]), str(csuite[f"c5_{i}_dtype"][0])
        np.testing.assert_array_equal(gpu.cdist_packed(pq, pc, k, dt), csuite[f"c5_{i}_out"])
        i += 1


@pytest.mark.parametrize("m", [1, 15, 16, 17, 31, 32, 33, 63, 64, 65, 127, 128, 129, 255, 256,
                               257, 511, 512, 513, 1000, 2047, 2048])
def test_length_boundaries_mixed_batch(gpu, m):
    rng = random.Random(m)
    A = [bytes(rng.randrange(256) for _ in range(rng.randrange(1, m + 1))) for _ in range(120)]
    B = [bytes(rng.randrange(256) for _ in range(rng.randrange(0, m + 30))) for _ in range(120)]
    # near-copies too, so trimming leaves long patterns in the middle
    for _ in range(40):
        a = bytearray(rng.randrange(4) for _ in range(m))
        b = bytearray(a)
        for _ in range(rng.randrange(1, 6)):
            b[rng.randrange(len(b))] = rng.randrange(4)
        A.append(bytes(a))
        B.append(bytes(b))
    pa, pb = oracle.pack(A), oracle.pack(B)
    for k in (None, 3):
        np.testing.assert_array_equal(gpu.pairwise_packed(pa, pb, k), oracle.pairs(pa, pb, k))
        np.testing.assert_array_equal(gpu.pairwise_packed(pb, pa, k), oracle.pairs(pb, pa, k))
    Q = A[:6] + [A[-1]]
    np.testing.assert_array_equal(gpu.cdist_packed(oracle.pack(Q), pb), oracle.cross(oracle.pack(Q), pb))


def test_zero_bytes_vs_padding(gpu):
    rng = random.Random(7)
    A = [bytes(rng.choice(b"\x00\x01") for _ in range(rng.randrange(1, 300))) for _ in range(600)]
    B = [bytes(rng.choice(b"\x00\x01") for _ in range(rng.randrange(0, 320))) for _ in range(600)]
    pa, pb = oracle.pack(A), oracle.pack(B)
    np.testing.assert_array_equal(gpu.pairwise_packed(pa, pb), oracle.pairs(pa, pb))
    pq = oracle.pack(A[:20])
    np.testing.assert_array_equal(gpu.cdist_packed(pq, pb), oracle.cross(pq, pb))


@pytest.mark.parametrize("k", [0, 1, 2, 5, 17, 100])
def test_threshold_and_dtypes(gpu, k):
    rng = np.random.default_rng(k)
    alph = np.frombuffer(b"ACGT\x00", dtype=np.uint8)
    a = W.random_strings(rng, rng.integers(0, 700, 3000), alph)
    b = W.mutate(rng, a, rng.uniform(0, 0.2, 3000), alph)
    exact = oracle.pairs(a, b)
    for dt in ("int32", "uint16", "uint8"):
        got = gpu.pairwise_packed(a, b, max_dist=k, dtype=dt)
        np.testing.assert_array_equal(got, oracle.saturate(np.minimum(exact, k + 1), dt))
    q = W.take(a, np.arange(40))
    c = W.take(b, np.arange(700))
    ex = oracle.cross(q, c)
    for dt in ("int32", "uint8"):
        np.testing.assert_array_equal(gpu.cdist_packed(q, c, k, dt),
                                      oracle.saturate(np.minimum(ex, k + 1), dt))


def test_return_device_and_empty(gpu):
    from editdist_bench_gb300 import DeviceArray
    r = gpu.cdist(["abc"], ["abd", "x"], return_device=True)
    assert isinstance(r, DeviceArray) and r.get().tolist() == [[1, 3]]
    assert r.shape == (1, 2) and r.__cuda_array_interface__["data"][0] != 0
    assert r.reshape(-1).get().tolist() == [1, 3]
    p = gpu.pairwise(["kitten", ""], ["sitting", "abc"], dtype=np.uint8, return_device=True)
    assert p.dtype == np.uint8 and p.get().tolist() == [3, 3]
    assert gpu.pairwise([], []).shape == (0,)
    assert gpu.cdist([], ["a"]).shape == (0, 1)
    assert gpu.cdist(["a"], []).shape == (1, 0)
    assert gpu.pairwise([], [], return_device=True).shape == (0,)
    assert gpu.cdist([], ["a"], return_device=True).get().shape == (0, 1)


def test_errors(gpu):
    with pytest.raises(ValueError):
        gpu.pairwise(["a"], ["a", "b"])
    with pytest.raises(ValueError):
        gpu.pairwise(["ok"], ["ā"])
    with pytest.raises(TypeError):
        gpu.pairwise(["ok"], [3])
    with pytest.raises(ValueError):
        gpu.cdist(["a"], ["b"], max_dist=-1)
    with pytest.raises(ValueError):
        gpu.cdist(["a"], ["b"], dtype=np.float32)
    # corrupt offsets are rejected by the device checks, not read out of range
    buf = np.frombuffer(b"abcdef", dtype=np.uint8)
    bad = np.array([0, 4, 2, 6], dtype=np.int64)
    good = np.array([0, 2, 4, 6], dtype=np.int64)
    with pytest.raises(ValueError):
        gpu.pairwise_packed((buf, bad), (buf, good))
    # the context stays usable after an error
    assert gpu.pairwise(["ab"], ["ac"]).tolist() == [1]


def test_generators_and_str_bytes_mix(gpu):
    P = [("kitten", "sitting"), (b"abc", "abd"), ("caf\xe9", b"cafe")]
    got = gpu.pairwise((p[0] for p in P), (p[1] for p in P))
    assert got.tolist() == [3, 1, 1]


def test_resident_batches_repeat(gpu):
    rng = np.random.default_rng(3)
    a = W.random_strings(rng, rng.integers(0, 400, 5000))
    b = W.mutate(rng, a, 0.08)
    batch = gpu.PairsBatch(a, b)
    exact = oracle.pairs(a, b)
    for k, dt in ((None, "int32"), (2, "uint8"), (9, "uint16"), (None, "int32")):
        out = batch.run(batch.alloc(dt), max_dist=k)
        want = exact if k is None else np.minimum(exact, k + 1)
        np.testing.assert_array_equal(out.get(), oracle.saturate(want, dt))
    q = W.take(a, np.arange(50))
    s = gpu.SearchBatch(q, b)
    ex = oracle.cross(q, b)
    for k, dt in ((None, "int32"), (4, "uint8"), (None, "uint16")):
        out = s.run(s.alloc(dt), max_dist=k)
        want = ex if k is None else np.minimum(ex, k + 1)
        np.testing.assert_array_equal(out.get(), oracle.saturate(want, dt))
    gpu.synchronize()


# ---- full benchmark sizes: exact where the oracle is fast enough, else
#      size-independent properties plus sampled rows -----------------------------
def test_config1_full(gpu):
    w = W.config1()
    np.testing.assert_array_equal(gpu.pairwise_packed(w.a, w.b), oracle.pairs(w.a, w.b, threads=8))


def test_config2_full_properties(gpu):
    w = W.config2()
    d32 = gpu.cdist_packed(w.q, w.c)
    d8 = gpu.cdist_packed(w.q, w.c, max_dist=2, dtype="uint8")
    # max_dist + uint8 output is exactly the capped exact matrix, everywhere
    np.testing.assert_array_equal(d8, np.minimum(d32, 3).astype(np.uint8))
    rows = np.random.default_rng(0).choice(w.nq, 6, replace=False)
    sub = W.take(w.q, rows)
    np.testing.assert_array_equal(d32[rows], oracle.cross(sub, w.c, threads=6))
    # the max_dist=2 run against the oracle directly (its own exit rule)
    rows8 = np.random.default_rng(1).choice(w.nq, 16, replace=False)
    np.testing.assert_array_equal(d8[rows8], oracle.saturate(oracle.cross(W.take(w.q, rows8), w.c, 2, threads=8),
                                                             "uint8"))
    # every planted choice is within 3% mutation of some query: its row minimum is small
    assert (d32.min(axis=0) <= 64).all()


def test_config3_full(gpu):
    w = W.config3()
    got = gpu.pairwise_packed(w.a, w.b, max_dist=8, dtype="uint8")
    np.testing.assert_array_equal(got, oracle.saturate(oracle.pairs(w.a, w.b, 8, threads=8), "uint8"))


def test_symmetry_property(gpu):
    rng = np.random.default_rng(9)
    q = W.random_strings(rng, rng.integers(0, 600, 300))
    d = gpu.cdist_packed(q, q)
    np.testing.assert_array_equal(d, d.T)
    assert (np.diag(d) == 0).all()


# ---- work order: every schedule gives identical results ----------------------
@pytest.mark.parametrize("sched", ["auto", "plain"])
def test_thresholded_search_schedules(gpu, sched):
    rng = np.random.default_rng(31)
    # wide and narrow length spreads, empty strings, planted near-copies
    q = W.concat(W.random_strings(rng, rng.integers(0, 300, 60)), W.random_strings(rng, [0, 1, 64, 65, 512]))
    c = W.concat(W.mutate(rng, W.take(q, rng.integers(0, 65, 300)), 0.05),
                 W.random_strings(rng, rng.integers(0, 320, 1500)), W.random_strings(rng, [0, 0, 7]))
    gpu.set_schedule(sched)
    try:
        for k, dt in ((0, "int32"), (2, "uint8"), (7, "uint16"), (40, "uint8"), (300, "int32"), (1000, "uint8")):
            got = gpu.cdist_packed(q, c, max_dist=k, dtype=dt)
            want = oracle.saturate(oracle.cross(q, c, k), dt)
            np.testing.assert_array_equal(got, want, err_msg=f"{sched} k={k} {dt}")
        # odd output sizes exercise the fill's unaligned head and tail
        q3, c3 = W.take(q, [1, 2, 3]), W.take(c, np.arange(997))
        np.testing.assert_array_equal(gpu.cdist_packed(q3, c3, 3, "uint8"),
                                      oracle.saturate(oracle.cross(q3, c3, 3), "uint8"))
    finally:
        gpu.set_schedule("auto")


def test_thresholded_search_resident_repeat(gpu):
    """The survivor plan is rebuilt per run: different k on one resident batch."""
    rng = np.random.default_rng(8)
    q = W.random_strings(rng, rng.integers(90, 130, 40))
    c = W.concat(W.mutate(rng, W.take(q, rng.integers(0, 40, 100)), 0.04),
                 W.random_strings(rng, rng.integers(80, 140, 2000)))
    s = gpu.SearchBatch(q, c)
    for k, dt in ((4, "uint8"), (0, "uint8"), (12, "int32"), (4, "uint8")):
        out = s.run(s.alloc(dt), max_dist=k).get()
        np.testing.assert_array_equal(out, oracle.saturate(oracle.cross(q, c, k), dt))


@pytest.mark.parametrize("sched", ["auto", "plain"])
def test_pairs_schedules(gpu, sched):
    rng = np.random.default_rng(77)
    alph = np.frombuffer(b"ACGTN", dtype=np.uint8)
    a = W.concat(W.random_strings(rng, rng.integers(0, 400, 6000), alph),
                 W.random_strings(rng, [0, 1, 64, 65, 128, 129, 2048], alph))
    b = W.mutate(rng, a, rng.uniform(0, 0.3, len(a[1]) - 1), alph)
    gpu.set_schedule(sched)
    try:
        for k, dt in ((None, "int32"), (0, "uint8"), (8, "uint8"), (30, "uint16"), (500, "int32")):
            got = gpu.pairwise_packed(a, b, max_dist=k, dtype=dt)
            np.testing.assert_array_equal(got, oracle.saturate(oracle.pairs(a, b, k), dt),
                                          err_msg=f"{sched} k={k}")
    finally:
        gpu.set_schedule("auto")


def test_pairs_exit_column_log(gpu):
    """The logged column counts: 0 for pairs settled by the length gap or an
    empty pattern, the trimmed text length without max_dist, at most the
    text length otherwise (the banded loop's exit may fire before the
    reference's bottom-row rule; only the values must agree)."""
    import ctypes
    from editdist_bench_gb300 import _lib
    rng = np.random.default_rng(5)
    a = W.random_strings(rng, rng.integers(0, 300, 4000))
    b = W.mutate(rng, a, rng.uniform(0, 0.3, 4000))
    batch = gpu.PairsBatch(a, b)
    ctx = _lib.context()
    for k in (None, 6):
        out = batch.alloc("int32")
        log = batch.alloc("int32")
        ctx.check(ctx.lib.blg_pairs_run_logged(ctx.h, batch.h, -1 if k is None else k, 0, out.ptr, log.ptr))
        cols = log.get()
        d, m_, n_, ocols = oracle.pairs_trace(a, b, k)
        np.testing.assert_array_equal(out.get(), d)
        assert (cols <= n_).all()
        settled = (m_ == 0) | (np.abs(n_ - m_) > (k if k is not None else 1 << 30))
        assert (cols[settled] == 0).all()
        if k is None:
            np.testing.assert_array_equal(cols[m_ > 0], n_[m_ > 0])


def test_problem_batch_graph(gpu):
    """Many cdist problems in one persistent launch, replayed from a CUDA graph:
    thresholded and exact problems, every dtype, empty problems, and a problem
    with queries longer than 256 (run per problem inside the same graph)."""
    rng = np.random.default_rng(55)
    probs = [(p.q, p.c, p.max_dist, p.dtype) for p in W.config5(n_problems=10, scale=1 / 128, seed=9)]
    probs.append((W.random_strings(rng, rng.integers(0, 200, 7)), W.random_strings(rng, rng.integers(0, 220, 900)),
                  None, "int32"))
    probs.append((W.random_strings(rng, [300, 20]), W.random_strings(rng, rng.integers(250, 330, 400)), 6, "uint8"))
    probs.append((W.random_strings(rng, []), W.random_strings(rng, [3, 4]), 2, "uint8"))
    batch = gpu.ProblemBatch(probs)
    for _ in range(2):                                   # capture, then replay
        outs = batch.run()
        gpu.synchronize()
        for (pq, pc, k, dt), o in zip(probs, outs):
            np.testing.assert_array_equal(o.get(), oracle.saturate(oracle.cross(pq, pc, k), dt))
    got = gpu.cdist_batch(probs[:3], return_device=False)
    for (pq, pc, k, dt), o in zip(probs[:3], got):
        np.testing.assert_array_equal(o, oracle.saturate(oracle.cross(pq, pc, k), dt))


def test_gram_filter_repeats_and_saturation(gpu):
    """The survivor filter's 4-gram counts saturate at 255 per bin: long runs
    of one symbol, periodic strings and their near-copies (distance small,
    counts far past 255) must keep their exact thresholded distances."""
    rng = np.random.default_rng(88)
    base = [b"A" * 500, b"AC" * 250, b"ACGT" * 125, b"AAAAC" * 100, b"G" * 300 + b"T" * 200]
    q = oracle.pack(base)
    variants = []
    for s in base:
        for e in range(0, 10):
            t = bytearray(s)
            for _ in range(e):
                i = int(rng.integers(0, len(t)))
                op = int(rng.integers(0, 3))
                if op == 0:
                    t[i] = int(rng.choice(list(b"ACGT")))
                elif op == 1:
                    t.insert(i, int(rng.choice(list(b"ACGT"))))
                elif len(t) > 1:
                    del t[i]
            variants.append(bytes(t))
    c = W.concat(oracle.pack(variants), W.random_strings(rng, rng.integers(490, 510, 300)))
    for k in (0, 3, 8, 31):
        for dt in ("uint8", "int32"):
            np.testing.assert_array_equal(gpu.cdist_packed(q, c, max_dist=k, dtype=dt),
                                          oracle.saturate(oracle.cross(q, c, k), dt), err_msg=f"k={k} {dt}")
