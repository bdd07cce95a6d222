"""GPU parity: the CUDA path, called through the C ABI, against the oracle and the reference's
own outputs (golden fixtures)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, load_golden
from efanna_gb300 import datasets, io

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


# ---------------------------------------------------------------------------------- distances
@pytest.mark.parametrize("d", [1, 3, 32, 100, 128, 960])
def test_l2_pairs_integer_exact(efg, oracle_lib, d):
    rng = np.random.default_rng(d)
    n, m = 500, 4000
    x = rng.integers(0, 256, (n, d)).astype(np.float32)
    ld = (d + 3) // 4 * 4
    xp = np.zeros((n, ld), np.float32)
    xp[:, :d] = x
    ia = rng.integers(0, n, m).astype(np.uint32)
    ib = rng.integers(0, n, m).astype(np.uint32)
    X, A, B = _dev(xp), _dev(ia), _dev(ib)
    out = torch.zeros(m, dtype=torch.float32, device="cuda")
    efg.l2_pairs_device(X.data_ptr(), n, d, ld, A.data_ptr(), B.data_ptr(), m, out.data_ptr())
    torch.cuda.synchronize()
    exact = ((x[ia].astype(np.int64) - x[ib].astype(np.int64)) ** 2).sum(1).astype(np.float32)
    assert np.array_equal(out.cpu().numpy(), exact)
    assert np.array_equal(oracle_lib.l2_pairs(x, ia, ib, "scalar"), exact)


@pytest.mark.parametrize("d", [32, 128, 960])
def test_l2_pairs_float_within_1e6_relative(efg, oracle_lib, d):
    x = datasets.mixture_unit(400, d, block=16 if d % 16 == 0 else d) if d % 16 == 0 else \
        np.random.default_rng(1).random((400, d), dtype=np.float32)
    rng = np.random.default_rng(2)
    m = 3000
    ia = rng.integers(0, 400, m).astype(np.uint32)
    ib = rng.integers(0, 400, m).astype(np.uint32)
    X, A, B = _dev(x), _dev(ia), _dev(ib)
    out = torch.zeros(m, dtype=torch.float32, device="cuda")
    efg.l2_pairs_device(X.data_ptr(), 400, d, d, A.data_ptr(), B.data_ptr(), m, out.data_ptr())
    torch.cuda.synchronize()
    g = out.cpu().numpy().astype(np.float64)
    for order in ("avx", "scalar"):
        r = oracle_lib.l2_pairs(x, ia, ib, order).astype(np.float64)
        tol = 1e-6 * np.abs(r) + 1e-30
        assert np.all(np.abs(g - r) <= tol), (order, np.max(np.abs(g - r) / np.maximum(r, 1e-30)))


@pytest.mark.parametrize("k,exclude", [(1, False), (10, True), (100, False)])
def test_brute_force_knn_exact(efg, k, exclude):
    x = datasets.mixture_u8(5000, 64, seed=4)
    q = x[:300] if exclude else datasets.mixture_u8(300, 64, seed=4, queries=True)
    X, Q = _dev(x), _dev(q)
    ids = torch.zeros((300, k), dtype=torch.int32, device="cuda")
    dist = torch.zeros((300, k), dtype=torch.float32, device="cuda")
    efg.brute_force_knn_device(X.data_ptr(), 5000, 64, 64, Q.data_ptr(), 300, 64, k, ids.data_ptr(),
                               dist.data_ptr(), exclude_self=exclude)
    torch.cuda.synchronize()
    xd, qd = x.astype(np.int64), q.astype(np.int64)
    D = ((qd[:, None, :] - xd[None, :, :]) ** 2).sum(2).astype(np.float64)
    if exclude:
        D[np.arange(300), np.arange(300)] = np.inf
    order = np.lexsort((np.broadcast_to(np.arange(5000), D.shape), D), axis=1)[:, :k]
    assert np.array_equal(ids.cpu().numpy(), order.astype(np.int32))
    assert np.array_equal(dist.cpu().numpy(), np.take_along_axis(D, order, 1).astype(np.float32))


# ---------------------------------------------------------------------------------- search
@pytest.mark.parametrize("case", ["small_d32", "mid_d128"])
def test_search_matches_reference_results(efg, case):
    """Same trees and graph files as the reference's efanna_search -> identical result ids."""
    g = load_golden(case)
    x = g["base"].astype(np.float32)
    q = g["queries"].astype(np.float32)
    st, se, pool, ext, k = [int(v) for v in g["search_params"]]
    idx = efg.Index(x, efg.IndexParams(trees=8))
    idx.load_trees(os.path.join(GOLDEN, case + ".trees"))
    idx.load_graph(os.path.join(GOLDEN, case + ".graph"))
    idx.set_search_params(se, pool, ext, st)
    res = idx.knn_search(k, q)
    assert np.array_equal(res, g["results"])
    s = idx.search_stats()
    assert s.queries == q.shape[0] and s.distance_evals >= pool * q.shape[0]


def test_search_device_api_and_evals_match_oracle(efg, oracle_lib, tmp_path):
    O = oracle_lib
    g = load_golden("mid_d128")
    x = g["base"].astype(np.float32)
    q = g["queries"].astype(np.float32)
    forest = O.Forest.load(os.path.join(GOLDEN, "mid_d128.trees"))
    gp, gi = io.read_graph_csr(os.path.join(GOLDEN, "mid_d128.graph"))
    for (ep, pool, ext, k, trees) in [(4, 600, 100, 10, 8), (2, 300, 300, 1, 4), (0, 100, 10, 20, 8),
                                      (3, 1000, 64, 64, 2)]:
        ref, ev = O.search(x, forest, gp, gi, q, k=k, epochs=ep, init_num=pool, extend_to=ext, trees=trees,
                           mode=O.CANON, threads=4, want_evals=True)
        idx = efg.Index(x, efg.IndexParams(trees=8))
        idx.load_trees(os.path.join(GOLDEN, "mid_d128.trees"))
        idx.load_graph(os.path.join(GOLDEN, "mid_d128.graph"))
        idx.set_search_params(ep, pool, ext, trees)
        res = idx.knn_search(k, q)
        assert np.array_equal(res, ref), (ep, pool, ext, k, trees)
        assert idx.search_stats().distance_evals == int(ev.sum())
        Q = _dev(q)
        out = torch.zeros((q.shape[0], k), dtype=torch.int32, device="cuda")
        idx.knn_search_device(k, Q.data_ptr(), q.shape[0], q.shape[1], out.data_ptr())
        torch.cuda.synchronize()
        assert np.array_equal(out.cpu().numpy(), ref)


def test_search_errors(efg):
    g = load_golden("small_d32")
    x = g["base"].astype(np.float32)
    idx = efg.Index(x, efg.IndexParams(trees=8))
    with pytest.raises(efg.EfannaError) as e:
        idx.knn_search(10, x[:4])
    assert e.value.code == efg.EFG_ERR_STATE
    idx.load_trees(os.path.join(GOLDEN, "small_d32.trees"))
    idx.load_graph(os.path.join(GOLDEN, "small_d32.graph"))
    idx.set_search_params(4, 100, 10, 9)
    with pytest.raises(efg.EfannaError) as e:
        idx.knn_search(10, x[:4])
    assert e.value.code == efg.EFG_ERR_TREE_COUNT
    idx.set_search_params(4, 5, 10, 8)
    with pytest.raises(efg.EfannaError) as e:
        idx.knn_search(10, x[:4])
    assert e.value.code == efg.EFG_ERR_ARG
    idx.set_search_params(4, 100, 10, 8)
    assert idx.knn_search(10, x[:0]).shape == (0, 10)


# ---------------------------------------------------------------------------------- trees
@pytest.mark.parametrize("n,d,trees,S,tns", [(3000, 32, 8, 10, 10), (4000, 128, 16, 10, 10), (2500, 20, 3, 4, 7)])
def test_trees_match_oracle_bytes(efg, oracle_lib, tmp_path, n, d, trees, S, tns):
    x = datasets.mixture_u8(n, d, seed=11)
    idx = efg.Index(x, efg.IndexParams(trees=trees, S=S, leaf_size=tns, L=max(30, S)))
    idx.build_trees()
    a = str(tmp_path / "g.trees")
    idx.save_trees(a)
    f = oracle_lib.Forest.build(x, trees, S=S, tns=tns, mode=oracle_lib.CANON, seed=1998)
    b = str(tmp_path / "o.trees")
    f.save(b, 10)
    assert open(a, "rb").read() == open(b, "rb").read()


def test_trees_float_data_match_oracle(efg, oracle_lib, tmp_path):
    x = datasets.mixture_unit(3000, 64, block=16)
    idx = efg.Index(x, efg.IndexParams(trees=4))
    idx.build_trees()
    idx.save_trees(str(tmp_path / "g.trees"))
    oracle_lib.Forest.build(x, 4, mode=oracle_lib.CANON).save(str(tmp_path / "o.trees"), 10)
    assert open(tmp_path / "g.trees", "rb").read() == open(tmp_path / "o.trees", "rb").read()


# ---------------------------------------------------------------------------------- NN-descent
def _state_diff(a, b):
    """First differing field of two NN-descent states (None if equal)."""
    for f in a.FIELDS:
        va, vb = getattr(a, f), getattr(b, f)
        if f in ("new_ids", "old_ids"):
            cnt = a.new_cnt if f == "new_ids" else a.old_cnt
            for i in range(a.n):
                if not np.array_equal(va[i, :cnt[i]], vb[i, :cnt[i]]):
                    return "%s row %d: %s vs %s" % (f, i, va[i, :cnt[i]], vb[i, :cnt[i]])
        elif not np.array_equal(va, vb):
            i = int(np.argwhere(va != vb)[0][0])
            return "%s row %d: %s vs %s" % (f, i, va[i], vb[i])
    return None


NND_CASES = [
    (3000, 32, dict(trees=8, merge_level=4, epochs=5, check=25, L=30, K=10, S=10)),
    (2500, 48, dict(trees=4, merge_level=3, epochs=4, check=40, L=20, K=8, S=6)),
    (2000, 16, dict(trees=6, merge_level=4, epochs=4, check=60, L=50, K=20, S=12)),
    (2000, 24, dict(trees=4, merge_level=3, epochs=3, check=10, L=12, K=5, S=4)),
    # pools of 101 and 151 entries: the merge's four- and eight-slot warp pools
    (2000, 16, dict(trees=4, merge_level=3, epochs=3, check=100, L=100, K=20, S=10)),
    (1500, 24, dict(trees=4, merge_level=3, epochs=3, check=150, L=150, K=20, S=10)),
]


@pytest.mark.parametrize("n,d,params", NND_CASES)
def test_nnd_init_and_iterations_match_oracle(efg, oracle_lib, n, d, params):
    O = oracle_lib
    x = datasets.mixture_u8(n, d, seed=7)
    p = O.make_params(K=params["K"], S=params["S"], L=params["L"], check_k=params["check"],
                      epochs=params["epochs"], trees=params["trees"], merge_level=params["merge_level"])
    forest = O.Forest.build(x, params["trees"], S=params["S"], mode=O.CANON)
    cap = max(p.L, 2 * p.S) + p.reverse_cap
    rc, st = O.nnd_init(x, forest, p, cap, O.CANON)
    assert rc == 0
    idx = efg.Index(x, efg.IndexParams(**params))
    idx.build_trees()
    gst = O.NNDState(x.shape[0], p.L, cap)
    idx.nnd_init(gst)
    assert _state_diff(st, gst) is None, ("init", _state_diff(st, gst))
    cur = st
    for it in range(params["epochs"]):
        nxt, pairs = O.nnd_iterate(x, cur, p, it, O.CANON)
        g = cur.copy()
        gp = idx.nnd_iterate(g, it)
        assert gp == pairs
        assert _state_diff(nxt, g) is None, (it, _state_diff(nxt, g))
        cur = nxt


@pytest.mark.parametrize("n,d,params", [
    (3000, 32, dict(trees=8, merge_level=4, epochs=8, check=25, L=30, K=10, S=10)),
    (4000, 128, dict(trees=8, merge_level=5, epochs=6, check=25, L=30, K=10, S=10)),
    (2500, 48, dict(trees=4, merge_level=3, epochs=4, check=40, L=20, K=8, S=6)),
    (2000, 16, dict(trees=6, merge_level=4, epochs=4, check=60, L=50, K=20, S=12)),
])
def test_full_build_matches_oracle(efg, oracle_lib, n, d, params):
    O = oracle_lib
    x = datasets.mixture_u8(n, d, seed=7)
    idx = efg.Index(x, efg.IndexParams(**params))
    idx.build_index()
    g = idx.graph()
    op = O.make_params(K=params["K"], S=params["S"], L=params["L"], check_k=params["check"],
                       epochs=params["epochs"], trees=params["trees"], merge_level=params["merge_level"])
    rc, gs, _, pairs = O.build_graph(x, op, O.CANON)
    assert rc == 0
    assert np.array_equal(g, gs.astype(g.dtype))
    assert idx.build_stats().join_pairs == pairs


def test_merge_level_error(efg):
    g = load_golden("small_d32")
    x = g["base"].astype(np.float32)
    idx = efg.Index(x, efg.IndexParams(trees=8, merge_level=8))
    with pytest.raises(efg.EfannaError) as e:
        idx.build_index()
    assert e.value.code == efg.EFG_ERR_MERGE_LEVEL
    assert idx.build_stats().max_merge_depth >= 0
    assert idx.graph_size() == 0
