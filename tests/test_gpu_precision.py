"""BF16 screening with FP32 re-rank (efg_set_search_precision) against the FP32 search.

On byte-valued data every BF16 row equals its FP32 row (integers up to 256 are exact in BF16) and
every squared distance is an integer below 2^24, so the BF16 walk makes the same decisions as
the FP32 walk and the ids must be identical.  On real-valued data the ids may differ where
rounding reorders near-ties; recall against exact neighbours must stay within 0.01 of FP32's.
"""
import numpy as np
import pytest

from efanna_gb300 import datasets

pytestmark = pytest.mark.gpu


def _exact_knn(x, q, k):
    x64, q64 = x.astype(np.float64), q.astype(np.float64)
    d = (q64 * q64).sum(1)[:, None] - 2 * q64 @ x64.T + (x64 * x64).sum(1)[None, :]
    return np.argsort(d, axis=1, kind="stable")[:, :k]


def _recall(res, gt):
    k = gt.shape[1]
    return np.mean([len(set(r[:k]) & set(g)) / k for r, g in zip(res, gt)])


def _index(efg, x, trees=8):
    idx = efg.Index(x, efg.IndexParams(trees=trees, merge_level=5, epochs=6, check=25, L=30, K=10, S=10))
    idx.build_index()
    return idx


@pytest.mark.parametrize("dim", [128, 13, 3, 40])
def test_bf16_ids_equal_fp32_on_byte_data(efg, dim):
    x = datasets.mixture_u8(6000, dim, seed=3).astype(np.float32)
    q = datasets.mixture_u8(300, dim, seed=3, queries=True).astype(np.float32)
    idx = _index(efg, x)
    for pt in [(4, 400, 80), (2, 60, 20), (6, 1500, 200)]:
        idx.set_search_params(*pt, 8)
        idx.set_search_precision("fp32")
        a = idx.knn_search(10, q)
        ev32 = idx.search_stats().distance_evals
        idx.set_search_precision("bf16")
        b = idx.knn_search(10, q)
        s = idx.search_stats()
        assert np.array_equal(a, b), pt
        assert s.distance_evals == ev32
        assert s.reranked == min(42, max(pt[2], 10))


def test_bf16_overflow_pass_equals_fp32(efg):
    """Large pools move visited sets to global memory (or through the overflow launch) in both
    modes."""
    x = datasets.mixture_u8(20000, 64, seed=4).astype(np.float32)
    q = datasets.mixture_u8(200, 64, seed=4, queries=True).astype(np.float32)
    idx = _index(efg, x)
    idx.set_search_params(8, 2000, 2000, 8)
    a = idx.knn_search(10, q)
    s32 = idx.search_stats()
    idx.set_search_precision("bf16")
    b = idx.knn_search(10, q)
    s16 = idx.search_stats()
    moved32 = s32.overflow_queries + s32.migrated_queries
    assert moved32 > 0 and s16.overflow_queries + s16.migrated_queries == moved32
    assert s16.kernel_launches == 2
    assert np.array_equal(a, b)


def test_bf16_recall_on_real_valued_data(efg):
    x = datasets.mixture_unit(12000, 100, block=20, seed=5)
    q = datasets.mixture_unit(300, 100, block=20, seed=5, queries=True)
    gt = _exact_knn(x, q, 10)
    idx = _index(efg, x)
    for pt in [(4, 300, 60), (6, 1200, 200)]:
        idx.set_search_params(*pt, 8)
        idx.set_search_precision("fp32")
        r32 = _recall(idx.knn_search(10, q), gt)
        idx.set_search_precision("bf16")
        r16 = _recall(idx.knn_search(10, q), gt)
        assert r16 >= r32 - 0.01, (pt, r32, r16)


def test_bf16_large_k_and_short_results(efg):
    x = datasets.mixture_u8(3000, 32, seed=6).astype(np.float32)
    q = datasets.mixture_u8(50, 32, seed=6, queries=True).astype(np.float32)
    idx = _index(efg, x)
    idx.set_search_params(3, 700, 700, 8)
    idx.set_search_precision("fp32")
    a = idx.knn_search(600, q)
    idx.set_search_precision("bf16")
    b = idx.knn_search(600, q)
    assert idx.search_stats().reranked == 700
    assert np.array_equal(a, b)


def test_precision_argument_errors(efg):
    x = datasets.mixture_u8(3000, 16, seed=7).astype(np.float32)
    idx = efg.Index(x, efg.IndexParams())
    with pytest.raises(ValueError):
        idx.set_search_precision("fp8")
    with pytest.raises(efg.EfannaError):
        efg._check(efg.lib().efg_set_search_precision(idx._h, 7))
