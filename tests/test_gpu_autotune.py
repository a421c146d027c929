"""The autotuner: it times launch shapes on this GPU, keeps sane values,
reloads them from its cache, and every result afterwards still equals the
oracle (shapes change only time)."""
import numpy as np
import pytest

import oracle
from editdist_bench_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def test_autotune_cache_and_exactness(gpu, tmp_path):
    path = str(tmp_path / "tune.txt")
    t = gpu.autotune(path)
    assert t["source"] == "timed"
    assert all(q in (4, 8, 16, 32, 64) for q in t["search_queries_per_cta"].values())
    assert t["survivor_ctas_per_sm"] in (2, 3, 4) and t["survivors_per_job"] in (2048, 4096)
    assert t["survivor_round_columns"] in (8, 16, 32)
    assert t["band_ctas_per_sm"] in (2, 3) and t["tile_shape"] in (1, 2, 3)
    # the max_dist axis: the wide buckets are tuned apart
    assert t["survivor_ctas_per_sm_k9_31"] in (2, 3, 4) and t["survivor_round_columns_k9_31"] in (8, 16, 32)
    assert t["band_ctas_per_sm_k16_31"] in (2, 3)
    t2 = gpu.autotune(path)                               # same device and library: loaded, not re-timed
    assert t2["source"] == "cache"
    assert {k: v for k, v in t2.items() if k != "source"} == {k: v for k, v in t.items() if k != "source"}
    rng = np.random.default_rng(12)
    q = W.random_strings(rng, rng.integers(0, 300, 40))
    c = W.concat(W.mutate(rng, W.take(q, rng.integers(0, 40, 200)), 0.03), W.random_strings(rng, rng.integers(0, 320, 3000)))
    # max_dist 3 and 8 run the narrow survivor shapes, 9, 12 and 31 the wide
    # ones (the bucket edges on both sides)
    for k, dt in ((None, "int32"), (3, "uint8"), (8, "uint8"), (9, "uint8"), (12, "uint16"), (31, "uint8")):
        np.testing.assert_array_equal(gpu.cdist_packed(q, c, k, dt), oracle.saturate(oracle.cross(q, c, k), dt))
    # the banded pairs solver: max_dist 8 and 15 narrow, 16 and 24 wide
    w = W.config3(n=50000, seed=5)
    for k in (8, 15, 16, 24):
        np.testing.assert_array_equal(gpu.pairwise_packed(w.a, w.b, k, "uint8"),
                                      oracle.saturate(oracle.pairs(w.a, w.b, k), "uint8"), err_msg=f"max_dist {k}")
