"""Search method 1 (getNeighbors_kgraph) on the GPU against the oracle's canonical restatement:
identical ids and distance-evaluation counts on the reference's own trees/graph files and on
GPU-built indexes, including the reference's enlargement of the stored pool size."""
import os

import numpy as np
import pytest
import torch

from conftest import GOLDEN, load_golden
from efanna_gb300 import datasets, io

pytestmark = pytest.mark.gpu

POINTS = [(8, 4, 400, 50, 10), (8, 4, 100, 50, 10), (8, 3, 600, 40, 20), (4, 2, 150, 100, 10),
          (8, 5, 200, 30, 5), (8, 1, 300, 7, 1), (2, 6, 64, 64, 33)]


def _golden_index(efg, case):
    g = load_golden(case)
    x = g["base"].astype(np.float32)
    idx = efg.Index(x, efg.IndexParams(trees=8))
    idx.load_trees(os.path.join(GOLDEN, case + ".trees"))
    idx.load_graph(os.path.join(GOLDEN, case + ".graph"))
    return g, x, g["queries"].astype(np.float32), idx


@pytest.mark.parametrize("case", ["small_d32", "mid_d128"])
def test_kgraph_matches_oracle_on_reference_files(efg, oracle_lib, case):
    O = oracle_lib
    g, x, q, _ = _golden_index(efg, case)
    forest = O.Forest.load(os.path.join(GOLDEN, case + ".trees"))
    gp, gi = io.read_graph_csr(os.path.join(GOLDEN, case + ".graph"))
    for st, ep, pool, ext, k in POINTS:
        _, _, _, idx = _golden_index(efg, case)
        ref, ev, pool2 = O.search_kgraph(x, forest, gp, gi, q, k=k, epochs=ep, init_num=pool, extend_to=ext,
                                         trees=st, mode=O.CANON, threads=4)
        idx.set_search_params(ep, pool, ext, st, -1, 1)
        res = idx.knn_search(k, q)
        assert np.array_equal(res, ref), (case, st, ep, pool, ext, k)
        assert idx.search_stats().distance_evals == int(ev.sum())
        # the second call runs with the enlarged pool size, as the reference's does
        ref2, _, _ = O.search_kgraph(x, forest, gp, gi, q, k=k, epochs=ep, init_num=pool2, extend_to=ext,
                                     trees=st, mode=O.CANON, threads=4)
        assert np.array_equal(idx.knn_search(k, q), ref2)
        idx.close()


def test_kgraph_close_to_reference_results(efg):
    """Against the reference's own kgraph ids (golden): ties ordered by id instead of by arrival
    change at most a few ids per thousand."""
    g, x, q, idx = _golden_index(efg, "mid_d128")
    kg = np.load(os.path.join(GOLDEN, "mid_d128_kgraph.npz"))
    for i, (st, ep, pool, ext, k) in enumerate(kg["points"]):
        idx.set_search_params(int(ep), int(pool), int(ext), int(st), -1, 1)
        res = idx.knn_search(int(k), q)
        assert np.mean(res == kg["first_%d" % i]) > 0.99


@pytest.mark.parametrize("K,dim", [(10, 64), (40, 24)])
def test_kgraph_gpu_built_index(efg, oracle_lib, K, dim):
    """GPU-built graph and trees (degree 40 exercises neighbour rows longer than a warp)."""
    O = oracle_lib
    x = datasets.mixture_u8(5000, dim, seed=11).astype(np.float32)
    q = datasets.mixture_u8(150, dim, seed=11, queries=True).astype(np.float32)
    idx = efg.Index(x, efg.IndexParams(trees=8, merge_level=4, epochs=6, L=max(30, K + 10), K=K))
    idx.build_index()
    gp, gi = idx.graph_csr()
    import tempfile
    with tempfile.TemporaryDirectory() as t:
        idx.save_trees(os.path.join(t, "t"))
        forest = O.Forest.load(os.path.join(t, "t"))
    for st, ep, pool, ext, k in [(8, 3, 500, 60, 10), (8, 4, 50, 50, 10), (4, 2, 800, 100, 50)]:
        idx.set_search_params(ep, pool, ext, st, -1, 1)
        res = idx.knn_search(k, q)
        ref, ev, _ = O.search_kgraph(x, forest, gp, gi, q, k=k, epochs=ep, init_num=pool, extend_to=ext,
                                     trees=st, mode=O.CANON, threads=4)
        assert np.array_equal(res, ref), (K, st, ep, pool, ext, k)
        assert idx.search_stats().distance_evals == int(ev.sum())


def test_kgraph_device_api_and_edges(efg, oracle_lib):
    O = oracle_lib
    g, x, q, idx = _golden_index(efg, "small_d32")
    forest = O.Forest.load(os.path.join(GOLDEN, "small_d32.trees"))
    gp, gi = io.read_graph_csr(os.path.join(GOLDEN, "small_d32.graph"))
    idx.set_search_params(3, 500, 40, 8, -1, 1)
    ref, _, _ = O.search_kgraph(x, forest, gp, gi, q, k=10, epochs=3, init_num=500, extend_to=40, trees=8,
                                mode=O.CANON)
    Q = torch.from_numpy(q).cuda()
    out = torch.zeros((q.shape[0], 10), dtype=torch.int32, device="cuda")
    idx.knn_search_device(10, Q.data_ptr(), q.shape[0], q.shape[1], out.data_ptr())
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), ref)
    # zero epochs: nothing is found (the reference emits an uninitialised slot; -1 here)
    idx.set_search_params(0, 100, 10, 8, -1, 1)
    assert np.all(idx.knn_search(5, q[:7]) == -1)
    # epochs * extend beyond n is refused (the reference's random fill would never end)
    idx.set_search_params(100, 100, 100, 8, -1, 1)
    with pytest.raises(efg.EfannaError):
        idx.knn_search(5, q[:3])
    # unknown method
    idx.set_search_params(2, 100, 10, 8, -1, 7)
    with pytest.raises(efg.EfannaError):
        idx.knn_search(5, q[:3])
