"""Deferred survivor results. With max_dist <= 31 the banded survivor kernel
fills the output with max_dist+1 itself (fill items taken between survivor
jobs) and sends every result <= max_dist to a list of 2^20 entries that a
scatter kernel stores after it; when more results than that turn up, a
repair launch runs the search again in place. Here a search and a batch
whose matrices are mostly matches (identical strings) overflow the list and
must still equal the oracle, and a smaller search checks the list path
itself against the oracle in every dtype.

Reference semantics: csrc/myers.c:101-143 (exit rules and caps),
bitlev/_common.py:25-29 (saturation).
"""
import numpy as np
import pytest

import oracle
from editdist_bench_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _mostly_equal(nq, n_same, n_rand, length, seed):
    """nq copies of one random DNA string as queries; choices: n_same more
    copies, then n_rand random strings (lengths length-3 .. length+3)."""
    rng = np.random.default_rng(seed)
    base = bytes(rng.choice(np.frombuffer(b"ACGT", np.uint8), length))
    rand = [bytes(rng.choice(np.frombuffer(b"ACGT", np.uint8), int(rng.integers(length - 3, length + 4))))
            for _ in range(n_rand)]
    return [base] * nq, [base] * n_same + rand


def _want_row(q, c, k, dtype):
    return oracle.saturate(oracle.cross(oracle.pack(q[:1]), oracle.pack(c), k), dtype)[0]


@pytest.mark.parametrize("dtype", ["uint8", "uint16", "int32"])
def test_list_overflow_repairs_resident_search(gpu, dtype):
    q, c = _mostly_equal(1024, 2048, 96, 40, seed=11)   # 2^21 results <= k: twice the list
    s = gpu.SearchBatch(oracle.pack(q), oracle.pack(c))
    got = s.run(s.alloc(dtype), max_dist=4).get()
    want = _want_row(q, c, 4, dtype)
    assert (want[:2048] == 0).all()
    np.testing.assert_array_equal(got, np.broadcast_to(want, got.shape))


def test_list_overflow_repairs_batch(gpu):
    q, c = _mostly_equal(1024, 2048, 96, 48, seed=12)
    q2, c2 = _mostly_equal(8, 16, 200, 100, seed=13)    # a small problem beside it
    batch = gpu.ProblemBatch([(oracle.pack(q), oracle.pack(c), 3, "uint16"),
                              (oracle.pack(q2), oracle.pack(c2), 5, "uint8")])
    for rep in range(2):                                 # the capture, then a replay
        outs = [o.get() for o in batch.run()]
        np.testing.assert_array_equal(outs[0], np.broadcast_to(_want_row(q, c, 3, "uint16"), outs[0].shape),
                                      err_msg=f"pass {rep}")
        np.testing.assert_array_equal(outs[1], np.broadcast_to(_want_row(q2, c2, 5, "uint8"), outs[1].shape),
                                      err_msg=f"pass {rep}")


@pytest.mark.parametrize("dtype", ["uint8", "uint16", "int32"])
def test_list_path_against_oracle(gpu, dtype):
    w = W.config4(nq=64, nc=1 << 14, seed=21)
    s = gpu.SearchBatch(w.q, w.c)
    got = s.run(s.alloc(dtype), max_dist=4).get()
    want = oracle.saturate(oracle.cross(w.q, w.c, 4), dtype)
    np.testing.assert_array_equal(got, want)
    assert (got <= 4).sum() > 0
