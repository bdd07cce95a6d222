"""BF16 screening with FP32 re-rank (efg_set_search_precision) against the FP32 search.

On byte-valued data every BF16 row equals its FP32 row (integers up to 256 are exact in BF16) and
every squared distance is an integer below 2^24, so the BF16 walk makes the same decisions as
the FP32 walk and the ids must be identical.  On real-valued data the ids may differ where
rounding reorders near-ties; recall against exact neighbours must stay within 0.01 of FP32's.
"""
import numpy as np
import torch
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
        idx.set_search_precision("fp4")
    with pytest.raises(efg.EfannaError):
        efg._check(efg.lib().efg_set_search_precision(idx._h, 7))


def _rel_errors(efg, idx, x, q, precision, m=256, seed=0):
    rng = np.random.default_rng(seed)
    ids = rng.integers(0, x.shape[0], (q.shape[0], m)).astype(np.uint32)
    Q = torch.from_numpy(np.ascontiguousarray(q, np.float32)).cuda()
    I = torch.from_numpy(ids.view(np.int32)).cuda()
    out = torch.zeros((q.shape[0], m), dtype=torch.float32, device="cuda")
    idx.screen_distances_device(precision, Q.data_ptr(), q.shape[0], q.shape[1], I.data_ptr(), m, out.data_ptr())
    torch.cuda.synchronize()
    d = out.cpu().numpy().astype(np.float64)
    x64, q64 = x.astype(np.float64), q.astype(np.float64)
    ref = ((x64[ids] - q64[:, None, :]) ** 2).sum(-1)
    rel = np.abs(d - ref) / np.maximum(ref, 1e-30)
    return rel.max(), rel.mean()


def test_distance_error_against_fp64(efg):
    """Each screening precision's squared-distance error against FP64: the unit-block GIST-like
    data (d = 960, values in [0, 1]) and the byte-valued data (d = 128)."""
    xu = datasets.mixture_unit(20000, 960, seed=9)
    qu = datasets.mixture_unit(64, 960, seed=9, queries=True)
    iu = efg.Index(xu, efg.IndexParams())
    e32 = _rel_errors(efg, iu, xu, qu, "fp32")
    e16 = _rel_errors(efg, iu, xu, qu, "bf16")
    e8 = _rel_errors(efg, iu, xu, qu, "fp8")
    print("d=960 unit data: relative error max/mean fp32 %.2e/%.2e bf16 %.2e/%.2e fp8 %.2e/%.2e" %
          (e32 + e16 + e8))
    assert e32[0] < 1e-5
    assert e16[1] < 5e-3 and e16[0] < 5e-2
    assert e8[1] < 5e-2 and e8[0] < 3e-1
    xb = datasets.mixture_u8(20000, 128, seed=9)
    qb = datasets.mixture_u8(64, 128, seed=9, queries=True)
    ib = efg.Index(xb, efg.IndexParams())
    assert _rel_errors(efg, ib, xb, qb, "fp32")[0] == 0.0  # integers: exact in any order
    assert _rel_errors(efg, ib, xb, qb, "bf16")[0] == 0.0  # bytes are exact in BF16
    e8b = _rel_errors(efg, ib, xb, qb, "fp8")
    print("d=128 byte data: fp8 relative error max/mean %.2e/%.2e" % e8b)
    assert 0 < e8b[1] < 5e-2


def test_screened_search_recall_at_100(efg):
    """The high-dimensional precision workload at small scale: d = 960 unit-block data, a K = 100
    graph (L = 200, check = 200), recall@100 of FP32, BF16 and FP8 screening with the FP32 re-rank."""
    x = datasets.mixture_unit(20000, 960, seed=13)
    q = datasets.mixture_unit(200, 960, seed=13, queries=True)
    gt = _exact_knn(x, q, 100)
    idx = efg.Index(x, efg.IndexParams(trees=8, merge_level=8, epochs=8, check=200, L=200, K=100, S=10))
    idx.build_index()
    idx.set_search_params(4, 1200, 200, 8)
    rec = {}
    for prec in ("fp32", "bf16", "fp8"):
        idx.set_search_precision(prec)
        res = idx.knn_search(100, q)
        rec[prec] = np.mean([len(set(r) & set(g)) / 100 for r, g in zip(res, gt)])
    print("recall@100: fp32 %.4f bf16 %.4f fp8 %.4f" % (rec["fp32"], rec["bf16"], rec["fp8"]))
    assert rec["bf16"] >= rec["fp32"] - 0.01
    assert rec["fp8"] >= rec["fp32"] - 0.03


def test_precision_workload_at_100k(efg):
    """The 960-d precision workload at N = 100,000 (unit-block generator, drawn on the GPU): K = 100
    graph (trees 8, ml 8, iter 8, L 200, check 200, S 10), 500 held-out queries, k = 100.  BF16
    screening with the FP32 re-rank keeps recall@100 within 0.005 of the FP32 search; FP8 within 0.03."""
    n, d, nq = 100_000, 960, 500
    X = datasets.mixture_unit_device(n, d, seed=5)
    Q = datasets.mixture_unit_device(nq, d, seed=5, queries=True)
    gt = torch.zeros((nq, 100), dtype=torch.int32, device="cuda")
    efg.brute_force_knn_device(X.data_ptr(), n, d, d, Q.data_ptr(), nq, d, 100, gt.data_ptr())
    torch.cuda.synchronize()
    gt = gt.cpu().numpy()
    idx = efg.Index.from_device(X.data_ptr(), n, d, d,
                                efg.IndexParams(trees=8, merge_level=8, epochs=8, check=200, L=200, K=100, S=10))
    idx.build_index()
    idx.set_search_params(4, 2000, 300, 8)
    out = torch.zeros((nq, 100), dtype=torch.int32, device="cuda")
    rec = {}
    for prec in ("fp32", "bf16", "fp8"):
        idx.set_search_precision(prec)
        idx.knn_search_device(100, Q.data_ptr(), nq, d, out.data_ptr())
        torch.cuda.synchronize()
        res = out.cpu().numpy()
        rec[prec] = np.mean([len(set(r.tolist()) & set(g.tolist())) / 100 for r, g in zip(res, gt)])
    print("N=100k d=960 recall@100: fp32 %.4f bf16 %.4f fp8 %.4f" % (rec["fp32"], rec["bf16"], rec["fp8"]))
    assert rec["fp32"] > 0.9
    assert rec["bf16"] >= rec["fp32"] - 0.005
    assert rec["fp8"] >= rec["fp32"] - 0.03
    idx.close()
