"""The short-pair tile kernel (pairwise under the automatic schedule when the
shorter string of at least 3 in 4 pairs is at most 32 bytes): bit-exact
against the oracle across tile boundaries, thresholds, dtypes, patterns
longer than 32 handed to the lane-spread consumer, and tiles whose byte span
is too large to stage (read in place)."""
import numpy as np
import pytest

import oracle
from editdist_bench_gb300 import workloads as W

pytestmark = pytest.mark.gpu

ALPH = np.frombuffer(b"ACGT\x00\xff", dtype=np.uint8)


def _short_pairs(rng, n, max_len=32, rate=(0.0, 0.3)):
    a = W.random_strings(rng, rng.integers(0, max_len + 1, n), ALPH)
    b = W.mutate(rng, a, rng.uniform(*rate, n), ALPH)
    return a, b


def _check(gpu, a, b, cases=((None, "int32"), (0, "uint8"), (1, "uint16"), (3, "uint8"), (31, "int32"),
                            (40, "uint8"))):
    exact = oracle.pairs(a, b)
    for k, dt in cases:
        want = oracle.saturate(exact if k is None else np.minimum(exact, k + 1), dt)
        np.testing.assert_array_equal(gpu.pairwise_packed(a, b, k, dt), want, err_msg=f"k={k} {dt}")
        np.testing.assert_array_equal(gpu.pairwise_packed(b, a, k, dt), want, err_msg=f"swapped k={k} {dt}")


@pytest.mark.parametrize("n", [1, 3, 511, 512, 513, 1027, 20000])
def test_tile_boundaries(gpu, n):
    rng = np.random.default_rng(n)
    _check(gpu, *_short_pairs(rng, n))


def test_tile_config1_shape_thresholds(gpu):
    w = W.config1(n=70001, seed=77)
    _check(gpu, w.a, w.b)


def test_tile_with_long_patterns_queued(gpu):
    """One pair in five has a pattern of 33..400 bytes: those leave the tile
    for the lane-spread consumer; the rest stay in the tile."""
    rng = np.random.default_rng(5)
    n = 9000
    lens = rng.integers(0, 33, n)
    long_i = rng.random(n) < 0.2
    lens[long_i] = rng.integers(33, 401, long_i.sum())
    a = W.random_strings(rng, lens, ALPH)
    b = W.mutate(rng, a, rng.uniform(0, 0.2, n), ALPH)
    _check(gpu, a, b)


def test_tile_span_too_large_reads_in_place(gpu):
    """A tile whose strings span more than the staging buffer (one text of
    40 KB among short pairs) is solved from global memory."""
    rng = np.random.default_rng(6)
    a, b = _short_pairs(rng, 3000)
    la, lb = np.diff(a[1]), np.diff(b[1])
    A = [a[0][a[1][i]:a[1][i + 1]].tobytes() for i in range(3000)]
    B = [b[0][b[1][i]:b[1][i + 1]].tobytes() for i in range(3000)]
    B[700] = bytes(rng.integers(0, 4, 40000).astype(np.uint8))
    B[2999] = bytes(rng.integers(0, 4, 20000).astype(np.uint8))
    pa, pb = oracle.pack(A), oracle.pack(B)
    assert la.max() <= 32 and lb.max() < 64
    _check(gpu, pa, pb, cases=((None, "int32"), (2, "uint8"), (31, "uint16")))


def test_tile_long_texts_smaller_tiles(gpu):
    """Short patterns against texts of 60..200 bytes: the tile shrinks so its
    span still stages."""
    rng = np.random.default_rng(8)
    n = 6000
    a = W.random_strings(rng, rng.integers(1, 33, n), ALPH)
    b = W.random_strings(rng, rng.integers(60, 201, n), ALPH)
    _check(gpu, a, b, cases=((None, "int32"), (5, "uint8"), (200, "uint16")))


def test_tile_offsets_with_base(gpu):
    """Offsets that do not start at 0 (a slice of a larger packed buffer)."""
    rng = np.random.default_rng(9)
    a, b = _short_pairs(rng, 4000)
    pad = np.frombuffer(b"xyz" * 7, dtype=np.uint8)
    a2 = (np.concatenate([pad, a[0]]), a[1] + len(pad))
    b2 = (np.concatenate([pad[:5], b[0]]), b[1] + 5)
    _check(gpu, a2, b2, cases=((None, "int32"), (4, "uint8")))


def test_tile_resident_repeat(gpu):
    rng = np.random.default_rng(10)
    a, b = _short_pairs(rng, 50000)
    batch = gpu.PairsBatch(a, b)
    exact = oracle.pairs(a, b)
    for k, dt in ((None, "int32"), (2, "uint8"), (None, "int32"), (7, "uint16")):
        out = batch.run(batch.alloc(dt), max_dist=k)
        want = exact if k is None else np.minimum(exact, k + 1)
        np.testing.assert_array_equal(out.get(), oracle.saturate(want, dt))


def test_tile_all_stage_shapes(gpu, tmp_path):
    """The tile kernel's staging shapes (an autotuned choice: one stage of 512
    pairs, two of 512, two of 256) give identical, exact results; each is
    forced through an edited tuning cache, on DNA (one row per byte) and on
    a 256-byte alphabet (nibble rows)."""
    path = tmp_path / "tune.txt"
    gpu.autotune(str(path))
    lines = path.read_text().splitlines()
    rng = np.random.default_rng(21)
    a, b = _short_pairs(rng, 30001)
    exact = oracle.pairs(a, b)
    full = np.arange(256, dtype=np.uint8)
    a2 = W.random_strings(rng, rng.integers(0, 33, 20003), full)
    b2 = W.mutate(rng, a2, 0.1, full)
    exact2 = oracle.pairs(a2, b2)
    for shape in (1, 2, 3):
        forced = tmp_path / f"tune{shape}.txt"
        forced.write_text("\n".join(l if not l.startswith("tile_shape") else f"tile_shape {shape}"
                                    for l in lines) + "\n")
        assert gpu.autotune(str(forced))["tile_shape"] == shape
        np.testing.assert_array_equal(gpu.pairwise_packed(a2, b2), exact2, err_msg=f"shape {shape}, 256 bytes")
        batch = gpu.PairsBatch(a2, b2)
        np.testing.assert_array_equal(batch.run(batch.alloc("int32")).get(), exact2, err_msg=f"shape {shape} resident")
        np.testing.assert_array_equal(gpu.pairwise_packed(a, b), exact)
        np.testing.assert_array_equal(gpu.pairwise_packed(a, b, 2, "uint8"),
                                      oracle.saturate(np.minimum(exact, 3), "uint8"))
    gpu.autotune(str(path))
