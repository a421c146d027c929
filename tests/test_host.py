"""Host-side logic without a GPU: bitlev's input semantics (checks, packing,
errors), the host build of the device primitives against the oracle, the
workload generators, and DeviceArray bookkeeping."""
import ctypes
import random

import numpy as np
import pytest

import oracle
from editdist_bench_gb300 import _build, workloads as W
from editdist_bench_gb300._common import check_dtype, check_k, convert, pack
from editdist_bench_gb300.device_array import DeviceArray


# ---- bitlev/_common.py semantics ------------------------------------------
def test_check_k_and_dtype():
    assert check_k(None) == -1 and check_k(0) == 0 and check_k(7) == 7
    assert check_k(2 ** 40) == 2 ** 30
    with pytest.raises(ValueError):
        check_k(-1)
    for dt in (np.int32, "uint16", np.uint8, "int32"):
        check_dtype(dt)
    for dt in (np.float32, np.int64, "int8"):
        with pytest.raises(ValueError):
            check_dtype(dt)
    np.testing.assert_array_equal(convert(np.array([0, 255, 256, 70000], np.int32), np.dtype(np.uint8)),
                                  [0, 255, 255, 255])
    np.testing.assert_array_equal(convert(np.array([0, 65535, 70000], np.int32), np.dtype(np.uint16)),
                                  [0, 65535, 65535])


# ---- packing (csrc/edpy.c:14-35, :200-224; tests/test_pack.py) -------------
@pytest.mark.parametrize("S", [[], [""], ["", ""], ["ab", "", "xyz"], ["\xff\x00\x80"],
                               ["q" * 1000] * 3, [b"by", "tes"], [b"x", b"", b"yz"]])
def test_pack_matches_oracle_pack(S):
    b1, o1 = pack(S)
    b2, o2 = oracle.pack(S)
    np.testing.assert_array_equal(o1, o2)
    assert bytes(b1[:o1[-1]]) == bytes(b2[:o2[-1]])
    assert len(b1) >= 1                       # never an empty buffer
    assert b1.dtype == np.uint8 and o1.dtype == np.int64


def test_pack_errors_and_generators():
    with pytest.raises(ValueError):
        pack(["ok", "ā"])                # above U+00FF
    with pytest.raises(ValueError):
        pack(["日本"])
    with pytest.raises(TypeError):
        pack(["ok", 3])
    with pytest.raises(TypeError):
        pack([1, "a"])
    with pytest.raises(TypeError):
        pack([b"a", bytearray(b"b")])        # bytes only, like PyBytes_Check
    b, o = pack(x for x in ["caf\xe9", "\xff\x00"])
    assert bytes(b[:o[-1]]) == b"caf\xe9\xff\x00" and o.tolist() == [0, 4, 6]


# ---- host build of the device primitives -----------------------------------
@pytest.fixture(scope="module")
def hostcheck():
    L = ctypes.CDLL(_build.build_hostcheck())
    for f in (L.blg_host_distance, L.blg_host_wavefront, L.blg_host_distance_halves):
        f.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_char_p, ctypes.c_int, ctypes.c_int,
                      ctypes.c_int]
        f.restype = ctypes.c_int
    L.blg_host_store.argtypes = [ctypes.c_int, ctypes.c_int]
    L.blg_host_band.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_char_p, ctypes.c_int, ctypes.c_int,
                                ctypes.c_int]
    L.blg_host_band_query.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_char_p, ctypes.c_int, ctypes.c_int]
    L.blg_host_band_blocks.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_char_p, ctypes.c_int, ctypes.c_int]
    L.blg_host_band_resume.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_char_p, ctypes.c_int, ctypes.c_int,
                                       ctypes.c_int]
    return L


def _one(a, b, k):
    return int(oracle.pairs(oracle.pack([a]), oracle.pack([b]), None if k < 0 else k)[0])


def test_hostcheck_edge_cases(hostcheck, known):
    for c in known["exact"]:
        a, b = c["a"].encode("latin-1"), c["b"].encode("latin-1")
        for trim in (0, 1):
            for f in (hostcheck.blg_host_distance, hostcheck.blg_host_wavefront,
                      hostcheck.blg_host_distance_halves):
                assert f(a, len(a), b, len(b), trim, -1) == c["d"]
                assert f(b, len(b), a, len(a), trim, -1) == c["d"]


@pytest.mark.parametrize("k", [-1, 0, 1, 2, 5, 8, 17, 100])
def test_hostcheck_random_threshold(hostcheck, k):
    rng = random.Random(1000 + k)
    for _ in range(300):
        m = rng.randrange(0, 700)
        a = bytes(rng.choice(b"ACGT\x00") for _ in range(m))
        b = bytearray(a)
        for _ in range(rng.randrange(0, 25)):
            i = rng.randrange(len(b) + 1)
            op = rng.randrange(3)
            if op == 0 and i < len(b): b[i] = rng.choice(b"ACGT")
            elif op == 1: b.insert(i, rng.choice(b"ACGT"))
            elif i < len(b): del b[i]
        b = bytes(b)
        want = _one(a, b, k)
        for trim in (0, 1):
            assert hostcheck.blg_host_distance(a, len(a), b, len(b), trim, k) == want
            assert hostcheck.blg_host_wavefront(a, len(a), b, len(b), trim, k) == want
            assert hostcheck.blg_host_distance_halves(a, len(a), b, len(b), trim, k) == want


@pytest.mark.parametrize("m", [1, 63, 64, 65, 127, 128, 129, 255, 256, 257, 511, 512, 513, 1000, 2048])
def test_hostcheck_word_boundaries(hostcheck, m):
    rng = random.Random(m)
    for _ in range(6):
        a = bytes(rng.randrange(256) for _ in range(m))
        b = bytes(rng.randrange(256) for _ in range(rng.randrange(max(0, m - 30), m + 30)))
        want = _one(a, b, -1)
        assert hostcheck.blg_host_distance(a, len(a), b, len(b), 1, -1) == want
        assert hostcheck.blg_host_wavefront(a, len(a), b, len(b), 0, -1) == want
        assert hostcheck.blg_host_distance_halves(a, len(a), b, len(b), 0, -1) == want


def test_hostcheck_store_saturation(hostcheck, known):
    s = known["saturation"]["store8"]
    assert [hostcheck.blg_host_store(d, 2) for d in s["in"]] == s["out"]
    assert [hostcheck.blg_host_store(d, 1) for d in (0, 65535, 65536, 10 ** 6)] == [0, 65535, 65535, 65535]
    assert hostcheck.blg_host_store(70000, 0) == 70000


# ---- workloads ----------------------------------------------------------------
def test_workloads_deterministic_and_shaped():
    a1, a2 = W.config1(n=2000), W.config1(n=2000)
    np.testing.assert_array_equal(a1.b[0], a2.b[0])
    assert (np.diff(a1.a[1]) == 32).all()
    w2 = W.config2(nq=64, nc=1000)
    assert w2.nq == 64 and w2.nc == 1000 and (np.diff(w2.q[1]) == 64).all()
    w3 = W.config3(n=3000)
    la = np.diff(w3.a[1])
    assert la.min() >= 8 and la.max() <= 256
    assert set(np.unique(w3.a[0][:w3.a[1][-1]]).tolist()) <= set(b"ACGTN")
    w4 = W.config4(nq=16, nc=2000)
    lq = np.diff(w4.q[1])
    assert lq.min() >= 100 and lq.max() <= 256
    probs = W.config5(n_problems=8, scale=0.01)
    assert len(probs) == 8 and all(0 <= p.max_dist <= 8 for p in probs)


def test_mutation_rate_bounds_distance():
    """At rate r each position edits with probability r, and every edit costs at
    most 1, so the distance never exceeds the number of edited positions."""
    rng = np.random.default_rng(5)
    a = W.random_strings(rng, np.full(3000, 50))
    b0 = W.mutate(np.random.default_rng(9), a, 0.0)
    np.testing.assert_array_equal(a[0][:a[1][-1]], b0[0][:b0[1][-1]])
    b = W.mutate(rng, a, 0.1)
    d = oracle.pairs(a, b)
    assert 3 <= d.mean() <= 7                  # ~ 50 * 0.1 edits, some cancel


def test_take_and_concat_roundtrip():
    S = [b"ab", b"", b"xyz", b"q" * 300]
    p = oracle.pack(S)
    assert W.unpack(W.take(p, [3, 0, 1])) == [S[3], S[0], S[1]]
    assert W.unpack(W.concat(p, W.take(p, [2]))) == S + [S[2]]


# ---- DeviceArray bookkeeping (no device memory touched) ----------------------
def test_device_array_shapes():
    d = DeviceArray(0, (6,), np.uint8, ctx=None)
    assert d.size == 6 and d.ndim == 1 and d.nbytes == 6 and len(d) == 6
    r = d.reshape(2, 3)
    assert r.shape == (2, 3) and r.reshape(-1).shape == (6,)
    cai = r.__cuda_array_interface__
    assert cai["shape"] == (2, 3) and cai["typestr"] == "|u1" and cai["version"] == 3
    with pytest.raises(ValueError):
        d.reshape(4, 2)
    e = DeviceArray(0, (0, 5), np.int32, ctx=None)
    assert e.size == 0 and e.reshape(5, 0).shape == (5, 0)


# ---- the banded loop (max_dist <= 31): exact min(d, k+1) for any lengths -----
@pytest.mark.parametrize("k", [0, 1, 2, 3, 5, 8, 13, 20, 31])
def test_band_matches_oracle(hostcheck, k):
    rng = random.Random(500 + k)
    for _ in range(400):
        m = rng.randrange(0, 420)
        al = rng.choice([b"AC", b"ACGT", b"ACGT\x00", bytes(range(256))])
        a = bytes(rng.choice(al) for _ in range(m))
        b = bytearray(a)
        for _ in range(rng.randrange(0, 3 * k + 4)):
            i = rng.randrange(len(b) + 1)
            op = rng.randrange(3)
            if op == 0 and i < len(b): b[i] = rng.choice(al)
            elif op == 1: b.insert(i, rng.choice(al))
            elif i < len(b): del b[i]
        b = bytes(b)
        if rng.random() < 0.5:
            a, b = b, a
        want = _one(a, b, k)
        assert hostcheck.blg_host_band(a, len(a), b, len(b), 1, k) == want
        assert hostcheck.blg_host_band(a, len(a), b, len(b), 0, k) == want
        assert hostcheck.blg_host_band_query(a, len(a), b, len(b), k) == want
        assert hostcheck.blg_host_band_blocks(a, len(a), b, len(b), k) == want


@pytest.mark.parametrize("k", [0, 4, 8, 31])
def test_band_stop_and_resume(hostcheck, k):
    """The thresholded search defers survivors still inside the band after
    4 (k + 4) columns: the state saved there and resumed with the window bits
    read from the unpadded Peq words gives the uninterrupted run's result,
    at every stop column (before, at and past the text's end)."""
    rng = random.Random(900 + k)
    for _ in range(150):
        m = rng.randrange(0, 300)
        al = rng.choice([b"ACGT", b"ACGTN", bytes(range(256))])
        a = bytes(rng.choice(al) for _ in range(m))
        b = bytearray(a)
        for _ in range(rng.randrange(0, 2 * k + 3)):
            i = rng.randrange(len(b) + 1)
            op = rng.randrange(3)
            if op == 0 and i < len(b): b[i] = rng.choice(al)
            elif op == 1: b.insert(i, rng.choice(al))
            elif i < len(b): del b[i]
        b = bytes(b)
        want = _one(a, b, k)
        assert hostcheck.blg_host_band_query(a, len(a), b, len(b), k) == want
        for stop in (0, 4, 4 * (k + 4), 64, 4 * (len(b) // 4), len(b) + 4 - len(b) % 4 if len(b) % 4 else len(b)):
            assert hostcheck.blg_host_band_resume(a, len(a), b, len(b), k, stop) == want, (a, b, k, stop)


def _gram_counts(s: bytes) -> np.ndarray:
    """Restatement of the device's binned 4-gram counts (gram_counts in
    blg_kernels.cuh): each 4-gram g = (b[i-3] << 24 | ... | b[i]) hashed by
    (g * 0x9E3779B1 mod 2^32) >> 28 into 16 bins, counters saturating at 255."""
    c = np.zeros(16, dtype=np.int64)
    for i in range(3, len(s)):
        g = (s[i - 3] << 24) | (s[i - 2] << 16) | (s[i - 1] << 8) | s[i]
        c[((g * 0x9E3779B1) & 0xFFFFFFFF) >> 28] += 1
    return np.minimum(c, 255)


def test_gram_count_bound_is_a_lower_bound():
    """The survivor filter's premise: sum over bins |count(x) - count(y)| / 8
    never exceeds the edit distance (an edit changes at most 4 grams of each
    string), on near-copies, unrelated strings, short strings and repeats."""
    import oracle
    rng = np.random.default_rng(17)
    a = W.concat(W.random_strings(rng, rng.integers(0, 120, 400)),
                 W.random_strings(rng, rng.integers(0, 40, 200), np.frombuffer(b"AC", dtype=np.uint8)))
    b = W.concat(W.mutate(rng, W.take(a, np.arange(300)), rng.uniform(0, 0.3, 300)),
                 W.random_strings(rng, rng.integers(0, 120, 300)))
    d = oracle.pairs(a, b)
    sa, sb = W.unpack(a), W.unpack(b)
    tight = 0
    for x, y, dist in zip(sa, sb, d):
        gd = int(np.abs(_gram_counts(x) - _gram_counts(y)).sum())
        assert gd <= 8 * dist, (x, y, dist, gd)
        tight += gd > 8 * (dist - 1)
    assert tight > 0            # the bound is reached often enough to filter


def test_native_pack_matches_python_pack():
    """The native packer (csrc/blg_pack.c) gives the same buffer, offsets and
    errors as the Python packer (the rules of csrc/edpy.c:14-35, 200-224)."""
    from editdist_bench_gb300 import _build, _common
    if _build.build_packer() is None:
        pytest.skip("no Python development headers: the numpy packer is the only one")
    import importlib
    importlib.reload(_common)
    assert _common._blgpack is not None
    rng = np.random.default_rng(3)
    cases = [[], [""], ["", b""], ["kitten", b"sitting", "caf\xe9", b"\x00\xff", "\x00"],
             [bytes(rng.integers(0, 256, int(n), dtype=np.uint8)) for n in rng.integers(0, 300, 500)],
             ["".join(chr(c) for c in rng.integers(0, 256, int(n))) for n in rng.integers(0, 50, 300)]]
    for seq in cases:
        got, want = _common.pack(seq), _common.pack_python(seq)
        np.testing.assert_array_equal(got[0], want[0])
        np.testing.assert_array_equal(got[1], want[1])
        assert len(got[0]) >= 1
    for bad, exc in ((["ok", "ā"], ValueError), (["ok", 3], TypeError), ([None], TypeError)):
        with pytest.raises(exc) as e1:
            _common.pack(bad)
        with pytest.raises(exc) as e2:
            _common.pack_python(bad)
        assert str(e1.value) == str(e2.value)


def test_windowed_gram_bound_is_a_lower_bound():
    """The pairs scheduler's feature: the 4-gram count distance of the first 64
    bytes of each (trimmed) string, over 16, never exceeds the distance."""
    import oracle
    rng = np.random.default_rng(19)
    a = W.random_strings(rng, rng.integers(0, 260, 600))
    b = W.concat(W.mutate(rng, W.take(a, np.arange(400)), rng.uniform(0, 0.4, 400)),
                 W.random_strings(rng, rng.integers(0, 260, 200)))
    d = oracle.pairs(a, b, trim=False)
    for x, y, dist in zip(W.unpack(a), W.unpack(b), d):
        gd = int(np.abs(_gram_counts(x[:64]) - _gram_counts(y[:64])).sum())
        assert gd <= 16 * dist, (x, y, dist, gd)
