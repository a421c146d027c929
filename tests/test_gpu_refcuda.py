"""The reference's own CUDA kernels (csrc/gpu_kernels.cu, compiled for sm_103a
from its sources and launched with bitlev/gpu.py's geometry by
oracle/ref_cuda.py) against the oracle and against this engine, on the same
GPU: the three agree bit for bit, which pins the oracle to the reference's GPU
path too and checks the harness bench.py times the reference with."""
import numpy as np
import pytest

import oracle
from oracle import ref_cuda
from editdist_bench_gb300 import gpu, workloads as W

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not ref_cuda.available(), reason="reference CUDA cubin not built here")]


@pytest.mark.parametrize("k,out8", [(-1, False), (3, True), (0, False)])
def test_reference_pairs_kernels_match_oracle_and_engine(k, out8):
    rng = np.random.default_rng(61)
    n = 5000
    a = W.random_strings(rng, rng.integers(0, 257, n))
    b = W.mutate(rng, a, rng.uniform(0, 0.3, n))
    keep = np.minimum(np.diff(a[1]), np.diff(b[1])) <= 256          # bitlev runs longer pairs on the CPU
    a, b = W.take(a, np.nonzero(keep)[0]), W.take(b, np.nonzero(keep)[0])
    dt = "uint8" if out8 else "int32"
    kk = None if k < 0 else k
    want = oracle.saturate(oracle.pairs(a, b, kk), dt)
    np.testing.assert_array_equal(ref_cuda.pairwise(a, b, k, out8), want)
    np.testing.assert_array_equal(gpu.pairwise_packed(a, b, kk, dt), want)


@pytest.mark.parametrize("k,out8", [(-1, False), (2, True)])
def test_reference_cross_kernels_match_oracle_and_engine(k, out8):
    rng = np.random.default_rng(62)
    q = W.random_strings(rng, rng.integers(0, 513, 40))
    c = W.concat(W.mutate(rng, q, 0.03), W.random_strings(rng, rng.integers(0, 300, 700)))
    dt = "uint8" if out8 else "int32"
    kk = None if k < 0 else k
    want = oracle.saturate(oracle.cross(q, c, kk), dt)
    np.testing.assert_array_equal(ref_cuda.cdist(q, c, k, out8), want)
    np.testing.assert_array_equal(gpu.cdist_packed(q, c, kk, dt), want)


def test_reference_kernels_on_config_shapes():
    """The benchmark shapes of L32 DNA pairs and the L64 DNA search, small counts."""
    w1 = W.config1(n=20000, seed=71)
    np.testing.assert_array_equal(ref_cuda.pairwise(w1.a, w1.b), oracle.pairs(w1.a, w1.b))
    w2 = W.config2(nq=16, nc=4096, seed=72)
    np.testing.assert_array_equal(ref_cuda.cdist(w2.q, w2.c), oracle.cross(w2.q, w2.c))
    np.testing.assert_array_equal(ref_cuda.cdist(w2.q, w2.c, 2, True),
                                  oracle.saturate(oracle.cross(w2.q, w2.c, 2), "uint8"))
