"""The oracle is pinned before it is trusted: its C restatement and its
Python ground truth must reproduce the reference's own answers (golden
fixtures generated by tests/golden/make_golden.py from the reference) and,
where the reference's C core is compiled here, agree with it directly."""
import random

import numpy as np
import pytest

import oracle
from oracle import build_oracle


def _enc(s):
    return s.encode("latin-1")


def test_known_answers_exact(known):
    for c in known["exact"]:
        a, b = _enc(c["a"]), _enc(c["b"])
        assert oracle.dp_distance(a, b) == c["d"], c["src"]
        assert oracle.myers_distance(a, b) == c["d"], c["src"]
        got = oracle.pairs(oracle.pack([a, b]), oracle.pack([b, a]))
        assert got.tolist() == [c["d"], c["d"]], c["src"]
        for trim in (False, True):
            assert oracle.pairs(oracle.pack([a]), oracle.pack([b]), trim=trim)[0] == c["d"]
        assert oracle.cross(oracle.pack([a]), oracle.pack([b]))[0, 0] == c["d"]


def test_known_answers_thresholded(known):
    for c in known["thresholded"]:
        a, b = _enc(c["a"]), _enc(c["b"])
        assert oracle.pairs(oracle.pack([a]), oracle.pack([b]), c["k"])[0] == c["d"], c["src"]
        assert oracle.cross(oracle.pack([a]), oracle.pack([b]), c["k"])[0, 0] == c["d"], c["src"]


def test_saturation(known):
    s = known["saturation"]
    Q, C = [_enc(x) for x in s["Q"]], [_enc(x) for x in s["C"]]
    for dt in ("int32", "uint8", "uint16"):
        assert oracle.cdist_api(Q, C, dtype=dt).tolist() == s[dt]
    assert oracle.pairwise_api([b"x" * 300], [b""], dtype=np.uint8)[0] == s["pair_x300_empty_uint8"]
    assert oracle.saturate(s["store8"]["in"], np.uint8).tolist() == s["store8"]["out"]


def test_random_suite_pairs(rsuite):
    pa = (rsuite["a_buf"], rsuite["a_off"])
    pb = (rsuite["b_buf"], rsuite["b_off"])
    for key, want in rsuite.items():
        if not key.startswith("pairs_"):
            continue
        _, kk, dt = key.split("_")
        k = None if kk == "knone" else int(kk[1:])
        got = oracle.saturate(oracle.pairs(pa, pb, k), dt)
        np.testing.assert_array_equal(got, want, err_msg=key)
        if k is None and dt == "int32":
            np.testing.assert_array_equal(oracle.pairs(pa, pb, k, trim=False), want)


def test_random_suite_cross(rsuite):
    pq = (rsuite["q_buf"], rsuite["q_off"])
    pc = (rsuite["c_buf"], rsuite["c_off"])
    for key, want in rsuite.items():
        if not key.startswith("cross_"):
            continue
        _, kk, dt = key.split("_")
        k = None if kk == "knone" else int(kk[1:])
        np.testing.assert_array_equal(oracle.saturate(oracle.cross(pq, pc, k), dt), want, err_msg=key)


def test_config_subsamples(csuite):
    for tag in ("c1", "c3"):
        pa = (csuite[f"{tag}_a_buf"], csuite[f"{tag}_a_off"])
        pb = (csuite[f"{tag}_b_buf"], csuite[f"{tag}_b_off"])
        k = None if tag == "c1" else 8
        dt = "int32" if tag == "c1" else "uint8"
        np.testing.assert_array_equal(oracle.saturate(oracle.pairs(pa, pb, k), dt), csuite[f"{tag}_out"])
    # the L32 pairs workload also against the reference's textbook DP on its 300-pair subsample
    pa = (csuite["c1_a_buf"], csuite["c1_a_off"])
    pb = (csuite["c1_b_buf"], csuite["c1_b_off"])
    np.testing.assert_array_equal(oracle.pairs(pa, pb)[:300], csuite["c1_dp300"])
    for tag, cases in (("c2", ((None, "int32"), (2, "uint8"))), ("c4", ((4, "uint8"),))):
        pq = (csuite[f"{tag}_q_buf"], csuite[f"{tag}_q_off"])
        pc = (csuite[f"{tag}_c_buf"], csuite[f"{tag}_c_off"])
        for k, dt in cases:
            want = csuite[f"{tag}_k{'none' if k is None else k}_{dt}"]
            np.testing.assert_array_equal(oracle.saturate(oracle.cross(pq, pc, k), dt), want)
    i = 0
    while f"c5_{i}_out" in csuite:
        pq = (csuite[f"c5_{i}_q_buf"], csuite[f"c5_{i}_q_off"])
        pc = (csuite[f"c5_{i}_c_buf"], csuite[f"c5_{i}_c_off"])
        k, dt = int(csuite[f"c5_{i}_k"][0]), str(csuite[f"c5_{i}_dtype"][0])
        np.testing.assert_array_equal(oracle.saturate(oracle.cross(pq, pc, k), dt), csuite[f"c5_{i}_out"])
        i += 1
    assert i > 0


@pytest.mark.parametrize("n", [1, 2, 31, 32, 33, 63, 64, 65, 127, 128, 129, 200])
def test_python_myers_matches_dp(n):
    rng = random.Random(n)
    for _ in range(25):
        a = "".join(rng.choice("ACGT") for _ in range(n))
        b = "".join(rng.choice("ACGT") for _ in range(rng.randint(0, n + 10)))
        assert oracle.myers_distance(a, b) == oracle.dp_distance(a, b)
        assert oracle.myers_distance(b, a) == oracle.dp_distance(a, b)


def test_trace_counts_columns():
    """The work record: gap exits and empty patterns process 0 columns,
    exact runs process every text column of the trimmed pair."""
    a = [b"AAAA", b"", b"ACGTACGT", b"ACGTTTTTACGT" * 3]
    b = [b"AAAAAAAAAAAA", b"ACG", b"ACGTACGA", b"ACGTACGT" * 4]
    d, m, n, cols = oracle.pairs_trace(oracle.pack(a), oracle.pack(b), 2)
    assert d[0] == 3 and cols[0] == 0                  # gap 8 > 2
    assert m[1] == 0 and cols[1] == 0
    assert d[2] == 1 and (m[2], n[2], cols[2]) == (1, 1, 1)
    d2, _, n2, cols2 = oracle.pairs_trace(oracle.pack(a), oracle.pack(b))
    assert (cols2 <= n2).all()


def test_threaded_drivers_agree():
    rng = np.random.default_rng(3)
    from editdist_bench_gb300 import workloads as W
    a = W.random_strings(rng, rng.integers(0, 200, 3000))
    b = W.mutate(rng, a, 0.1)
    for k in (None, 4):
        np.testing.assert_array_equal(oracle.pairs(a, b, k, threads=4), oracle.pairs(a, b, k))
    q = W.random_strings(rng, rng.integers(0, 150, 40))
    c = W.random_strings(rng, rng.integers(0, 150, 300))
    np.testing.assert_array_equal(oracle.cross(q, c, 3, threads=3), oracle.cross(q, c, 3))


@pytest.mark.skipif(not build_oracle.ref_available(), reason="reference checkout absent")
def test_against_reference_c_core():
    """Direct differential test: the reference's libmyers.so / gpucheck, compiled
    from its own sources, against the restatement on fresh random data."""
    build_oracle.build_ref()
    L = oracle.ref_libmyers()
    G = oracle.ref_gpucheck()
    rng = np.random.default_rng(11)
    from editdist_bench_gb300 import workloads as W
    alph = np.frombuffer(b"ACGT\x00\xff", dtype=np.uint8)
    a = W.random_strings(rng, rng.integers(0, 400, 4000), alph)
    b = W.mutate(rng, a, rng.uniform(0, 0.4, 4000), alph)
    n = 4000
    for k in (-1, 0, 1, 3, 8, 30):
        ref = np.empty(n, dtype=np.int32)
        assert L.ed_pairs_k(a[0], a[1], b[0], b[1], n, ref, 1, k) == 0
        np.testing.assert_array_equal(oracle.pairs(a, b, None if k < 0 else k), ref)
    q = W.take(a, np.arange(25))
    c = W.take(b, np.arange(300))
    ref = np.empty((25, 300), dtype=np.int32)
    assert L.ed_cross(q[0], q[1], 25, c[0], c[1], 300, ref) == 0
    np.testing.assert_array_equal(oracle.cross(q, c), ref)
    A, B = W.unpack(W.take(a, np.arange(500))), W.unpack(W.take(b, np.arange(500)))
    for x, y in zip(A, B):
        if min(len(x), len(y)) <= 256:
            for k in (-1, 2):
                want = oracle.pairs(oracle.pack([x]), oracle.pack([y]), None if k < 0 else k)[0]
                assert G.gpu_pair_distance_host(x, len(x), y, len(y), 1, k) == want
