"""Edge cases of the path against the oracle's canonical restatement: exact duplicates (distance
ties everywhere), dimensions that are not multiples of the vector widths, the smallest base the
build accepts, empty query batches, queries equal to base points, and graphs with rows of different
lengths (loaded from a file), and a device-side limit made to fire."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, load_golden
from efanna_gb300 import datasets, io

pytestmark = pytest.mark.gpu

P = dict(trees=4, merge_level=3, epochs=4, check=25, L=20, K=8, S=6)


def _oracle_params(O, p):
    return O.make_params(K=p["K"], S=p["S"], L=p["L"], check_k=p["check"], epochs=p["epochs"], trees=p["trees"],
                         merge_level=p["merge_level"], tns=p.get("leaf_size", 10))


def _build_and_check(efg, O, x, p):
    idx = efg.Index(x, efg.IndexParams(**p))
    idx.build_index()
    rc, gs, forest, _ = O.build_graph(x, _oracle_params(O, p), O.CANON)
    assert rc == 0
    assert np.array_equal(idx.graph(), gs.astype(np.uint32))
    return idx, forest, gs


def _search_check(efg, O, idx, forest, gs, x, q, pt, trees):
    gp, gi = O.graph_csr_from_dense(gs)
    idx.set_search_params(pt[0], pt[1], pt[2], trees)
    res = idx.knn_search(10, q)
    ref = O.search(x, forest, gp, gi, q, k=10, epochs=pt[0], init_num=pt[1], extend_to=pt[2], trees=trees,
                   mode=O.CANON, threads=4)
    assert np.array_equal(res, ref)
    return res


def test_exact_duplicates(efg, oracle_lib):
    """Every point three times: distance-0 ties in the join, the merge, the trees and the search."""
    O = oracle_lib
    base = datasets.mixture_u8(900, 24, seed=31)
    x = np.ascontiguousarray(np.repeat(base, 3, axis=0))
    idx, forest, gs = _build_and_check(efg, O, x, P)
    q = np.ascontiguousarray(x[::97][:30])  # queries that are base points
    res = _search_check(efg, O, idx, forest, gs, x, q, (4, 300, 60), 4)
    # a query equal to a base row finds that row's copies first (distance 0, ties by id)
    rows = np.arange(0, x.shape[0], 97)[:30]
    for r, row in zip(res, rows):
        copies = set(range(row - row % 3, row - row % 3 + 3))
        assert set(r[:3].tolist()) == copies


@pytest.mark.parametrize("d", [1, 3, 5, 17, 33])
def test_ragged_dimensions(efg, oracle_lib, d):
    O = oracle_lib
    x = datasets.mixture_u8(1500, d, seed=40 + d)
    q = datasets.mixture_u8(40, d, seed=40 + d, queries=True)
    p = dict(P, merge_level=2) if d == 1 else P
    idx, forest, gs = _build_and_check(efg, O, x, p)
    _search_check(efg, O, idx, forest, gs, x, q, (3, 200, 40), 4)


def test_smallest_base_and_pool_bounds(efg, oracle_lib):
    """n = 2S + 2, the smallest base the build accepts; a pool of the whole base."""
    O = oracle_lib
    p = dict(trees=2, merge_level=1, epochs=3, check=10, L=6, K=4, S=4, leaf_size=3)
    n = 2 * p["S"] + 2
    x = datasets.mixture_u8(n, 8, seed=50)
    q = datasets.mixture_u8(5, 8, seed=50, queries=True)
    idx, forest, gs = _build_and_check(efg, O, x, p)
    gp, gi = O.graph_csr_from_dense(gs)
    idx.set_search_params(2, n, 4, 2)
    ref = O.search(x, forest, gp, gi, q, k=n, epochs=2, init_num=n, extend_to=4, trees=2, mode=O.CANON)
    assert np.array_equal(idx.knn_search(n, q), ref)
    idx.set_search_params(2, n + 1, 4, 2)
    with pytest.raises(efg.EfannaError):
        idx.knn_search(5, q)
    with pytest.raises(efg.EfannaError):
        efg.Index(datasets.mixture_u8(n - 1, 8, seed=50), efg.IndexParams(**p))


def test_empty_batches(efg):
    x = datasets.mixture_u8(2000, 16, seed=60)
    idx = efg.Index(x, efg.IndexParams(**P))
    idx.build_index()
    empty = np.zeros((0, 16), np.float32)
    for method in (0, 1):
        idx.set_search_params(3, 200, 40, 4, -1, method)
        assert idx.knn_search(10, empty).shape == (0, 10)
    idx.set_search_params(3, 200, 40, 4)
    assert idx.knn_search_batch(empty, np.zeros((0, 4), np.int32), 10).shape == (0, 10)


def test_variable_degree_graph_from_file(efg, oracle_lib, tmp_path):
    """A graph file whose rows have different lengths: nnexp and kgraph read row pointers."""
    O = oracle_lib
    x = datasets.mixture_u8(2000, 16, seed=70)
    q = datasets.mixture_u8(60, 16, seed=70, queries=True)
    idx = efg.Index(x, efg.IndexParams(**P))
    idx.build_index()
    g = idx.graph()
    K = g.shape[1]
    rng = np.random.default_rng(1)
    # lengths K + a and K - a in pairs (the first row full): the file keeps n * (K + 1) words, which
    # is how the loader (like the reference's loadGraph) infers the row count from the first row
    lens = np.full(g.shape[0], K)
    for i in range(1, g.shape[0] - 1, 2):
        a = int(rng.integers(0, 4))
        lens[i], lens[i + 1] = K + a, K - a
    rows = [np.concatenate([g[i], g[(i + 1) % g.shape[0]]])[:lens[i]] for i in range(g.shape[0])]
    path = str(tmp_path / "var.graph")
    with open(path, "wb") as f:
        for r in rows:
            np.array([len(r)], np.uint32).tofile(f)
            r.astype(np.uint32).tofile(f)
    idx.load_graph(path)
    gp, gi = io.read_graph_csr(path)
    t = str(tmp_path / "t.trees")
    idx.save_trees(t)
    forest = O.Forest.load(t)
    for pt in [(3, 200, 40), (5, 500, 100)]:
        idx.set_search_params(pt[0], pt[1], pt[2], 4)
        ref = O.search(x, forest, gp, gi, q, k=10, epochs=pt[0], init_num=pt[1], extend_to=pt[2], trees=4,
                       mode=O.CANON, threads=4)
        assert np.array_equal(idx.knn_search(10, q), ref), pt
        idx.set_search_params(pt[0], pt[1], pt[2], 4, -1, 1)
        kref, _, _ = O.search_kgraph(x, forest, gp, gi, q, k=10, epochs=pt[0], init_num=pt[1], extend_to=pt[2],
                                     trees=4, mode=O.CANON, threads=4)
        assert np.array_equal(idx.knn_search(10, q), kref), pt


def test_candidate_buffer_overflow_returns_device_limit(efg):
    """A device-side limit made to fire without any fault: the candidate buffer bounded below what
    one expansion epoch appends (extend = pool = 600 over a degree-10 graph appends up to 6000
    candidates; the bound is clamped up to the pool and the descent frontier, under 1000 here).
    The kernel drops the extra candidates, sets its error word, and the call returns
    EFG_ERR_DEVICE_LIMIT; with the bound lifted the same index searches as before."""
    g = load_golden("mid_d128")
    x = g["base"].astype(np.float32)
    q = g["queries"].astype(np.float32)
    idx = efg.Index(x, efg.IndexParams(trees=8))
    idx.load_trees(os.path.join(GOLDEN, "mid_d128.trees"))
    idx.load_graph(os.path.join(GOLDEN, "mid_d128.graph"))
    idx.set_search_params(4, 600, 600, 8)
    before = idx.knn_search(10, q)
    idx.set_search_candidate_cap(1)
    with pytest.raises(efg.EfannaError) as e:
        idx.knn_search(10, q)
    assert e.value.code == efg.EFG_ERR_DEVICE_LIMIT and "candidate buffer overflow" in str(e.value)
    idx.set_search_candidate_cap(0)
    assert np.array_equal(idx.knn_search(10, q), before)
    idx.set_search_params(4, 600, 100, 8)  # 100 x 10 items per epoch fit a 1000-entry bound
    ref = idx.knn_search(10, q)
    idx.set_search_candidate_cap(1000)
    assert np.array_equal(idx.knn_search(10, q), ref)
    idx.close()
