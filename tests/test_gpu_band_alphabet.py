"""The pairs kernels' pattern rows have two layouts: one row per byte when
the pair set uses at most 15 distinct bytes, nibble rows otherwise -- in the
banded solver (max_dist <= 31, any lengths) and in the short-pair tile
kernel. A resident set picks the layout at upload from its bytes; a one-call
run scans its bytes on the stream and launches both variants, of which the
one that does not apply returns at once. Every alphabet size around the
limit (1, 2, 4, 15, 16, 17, 256 bytes), with bytes spread over the whole
0..255 range, gives the oracle's results on both routes.
Reference semantics: csrc/myers.c:101-143 (max_dist exits and caps)."""
import numpy as np
import pytest

import oracle
from editdist_bench_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _pairs(rng, alphabet, n):
    la = rng.integers(1, 300, n)
    a = W.random_strings(rng, la, alphabet)
    b = W.mutate(rng, a, rng.uniform(0.0, 0.12, n), alphabet)
    return a, b


@pytest.mark.parametrize("size", [1, 2, 4, 15, 16, 17, 256])
def test_band_alphabet_sizes(gpu, size):
    rng = np.random.default_rng(900 + size)
    alphabet = np.sort(rng.choice(256, size, replace=False)).astype(np.uint8)
    a, b = _pairs(rng, alphabet, 20000)
    for k in (0, 6, 31):
        want = oracle.saturate(oracle.pairs(a, b, k, threads=8), "uint8")
        np.testing.assert_array_equal(gpu.pairwise_packed(a, b, max_dist=k, dtype="uint8"), want,
                                      err_msg=f"one-call, {size} bytes, k={k}")
        batch = gpu.PairsBatch(a, b)
        out = batch.run(batch.alloc("uint8"), max_dist=k)
        np.testing.assert_array_equal(out.get(), want, err_msg=f"resident, {size} bytes, k={k}")


def test_band_alphabet_pipelined_chunks(gpu):
    """2^18 + 5 pairs: the one-call pipeline scans each chunk's bytes on its
    own; the chunks use different alphabets (DNA, then 200 bytes)."""
    rng = np.random.default_rng(950)
    n1 = (1 << 17)
    a1, b1 = _pairs(rng, np.frombuffer(b"ACGT", dtype=np.uint8), n1)
    a2, b2 = _pairs(rng, np.arange(20, 220, dtype=np.uint8), (1 << 17) + 5)
    a, b = W.concat(a1, a2), W.concat(b1, b2)
    want = oracle.saturate(oracle.pairs(a, b, 8, threads=16), "uint8")
    np.testing.assert_array_equal(gpu.pairwise_packed(a, b, max_dist=8, dtype="uint8"), want)


@pytest.mark.parametrize("size", [1, 4, 15, 16, 256])
def test_tile_alphabet_sizes(gpu, size):
    """Short pairs (at most 32 bytes, the tile kernel), exact and thresholded."""
    rng = np.random.default_rng(980 + size)
    alphabet = np.sort(rng.choice(256, size, replace=False)).astype(np.uint8)
    la = rng.integers(0, 33, 30000)
    a = W.random_strings(rng, la, alphabet)
    b = W.mutate(rng, a, rng.uniform(0.0, 0.2, 30000), alphabet)
    for k, dt in ((None, "int32"), (3, "uint8")):
        want = oracle.saturate(oracle.pairs(a, b, k, threads=8), dt)
        np.testing.assert_array_equal(gpu.pairwise_packed(a, b, max_dist=k, dtype=dt), want,
                                      err_msg=f"one-call, {size} bytes, k={k}")
        batch = gpu.PairsBatch(a, b)
        out = batch.run(batch.alloc(dt), max_dist=k)
        np.testing.assert_array_equal(out.get(), want, err_msg=f"resident, {size} bytes, k={k}")
