"""Batching form: per-query search parameters in one launch, the device-counter batch size and
captured search plans (CUDA graph replay, autotuned block size), each query's ids identical to the
oracle's search with that query's own parameters."""
import os

import numpy as np
import pytest
import torch

from conftest import GOLDEN, load_golden
from efanna_gb300 import io

pytestmark = pytest.mark.gpu

CHOICES = [(4, 600, 100, 10), (2, 300, 60, 1), (6, 1000, 150, 50), (0, 200, 20, 10), (3, 120, 120, 100),
           (5, 800, 80, 20)]


@pytest.fixture(scope="module")
def setup(efg, oracle_lib):
    O = oracle_lib
    g = load_golden("mid_d128")
    x = g["base"].astype(np.float32)
    q = g["queries"].astype(np.float32)
    forest = O.Forest.load(os.path.join(GOLDEN, "mid_d128.trees"))
    gp, gi = io.read_graph_csr(os.path.join(GOLDEN, "mid_d128.graph"))
    ref = {}
    for c in CHOICES:
        ep, pool, ext, k = c
        ref[c] = O.search(x, forest, gp, gi, q, k=k, epochs=ep, init_num=pool, extend_to=ext, trees=8, mode=O.CANON,
                          threads=4)
    idx = efg.Index(x, efg.IndexParams(trees=8))
    idx.load_trees(os.path.join(GOLDEN, "mid_d128.trees"))
    idx.load_graph(os.path.join(GOLDEN, "mid_d128.graph"))
    idx.set_search_params(4, 600, 100, 8)

    def oracle(qs):  # per-choice results for a batch (the short-pool random fill is keyed by batch row)
        return {c: O.search(x, forest, gp, gi, qs, k=c[3], epochs=c[0], init_num=c[1], extend_to=c[2], trees=8,
                            mode=O.CANON, threads=4) for c in CHOICES}
    yield idx, q, ref, oracle
    idx.close()


def _params(nq, seed):
    pick = np.random.default_rng(seed).integers(0, len(CHOICES), nq)
    return pick, np.array([CHOICES[i] for i in pick], np.int32)


def _check_rows(out, pick, ref):
    for r, i in enumerate(pick):
        k = CHOICES[i][3]
        assert np.array_equal(out[r, :k], ref[CHOICES[i]][r]), (r, CHOICES[i])
        assert np.all(out[r, k:] == -1)


def test_per_query_parameters_match_oracle(efg, setup):
    idx, q, ref, _ = setup
    pick, params = _params(q.shape[0], 0)
    out = idx.knn_search_batch(q, params, 100)
    _check_rows(out, pick, ref)
    # every query at one setting through the batch API equals the plain search
    same = np.tile(np.array([4, 600, 100, 10], np.int32), (q.shape[0], 1))
    assert np.array_equal(idx.knn_search_batch(q, same, 10), idx.knn_search(10, q))


def test_batch_device_counter(efg, setup):
    idx, q, ref, _ = setup
    pick, params = _params(q.shape[0], 1)
    Q = torch.from_numpy(q).cuda()
    P = torch.from_numpy(params).cuda()
    out = torch.full((q.shape[0], 100), -7, dtype=torch.int32, device="cuda")
    n = torch.tensor([73], dtype=torch.int32, device="cuda")
    idx.knn_search_batch_device(Q.data_ptr(), q.shape[0], q.shape[1], P.data_ptr(), (6, 1000, 150, 100),
                                out.data_ptr(), n.data_ptr())
    torch.cuda.synchronize()
    o = out.cpu().numpy()
    _check_rows(o[:73], pick[:73], ref)
    assert np.all(o[73:] == -7)  # queries past the device count are untouched


@pytest.mark.parametrize("calibrate", [False, True])
def test_search_plan_replays(efg, setup, calibrate):
    idx, q, _, oracle = setup
    plan = idx.search_plan(128, (6, 1000, 150, 100), calib=q[:64] if calibrate else None)
    assert plan.threads in ((256, 512) if calibrate else (0,))
    cfg = plan.config
    if calibrate:  # the autotuner's record (plan creation also checked that every variant gave the same ids)
        assert cfg["variants"] >= 2 and cfg["tuned_ms"] > 0
        assert cfg["ht_pct"] in (50, 100, 200) and cfg["ctas_per_sm"] in (0, 1)
    else:
        assert cfg == {"threads": 0, "ctas_per_sm": 0, "ht_pct": 0, "variants": 0, "tuned_ms": 0.0}
    rng = np.random.default_rng(2)
    for size in [1, 128, 37, 100]:
        rows = rng.choice(q.shape[0], size, replace=False)
        pick, params = _params(size, size)
        out = plan.run(q[rows], params)
        _check_rows(out, pick, oracle(q[rows]))
    with pytest.raises(efg.EfannaError):
        plan.run(q[:129], _params(129, 0)[1])
    plan.close()


def test_two_plans_in_flight(efg, setup):
    """Two plans of one index with batches in flight at once (own streams and scratch; a batch
    larger than a CTA wave so the overflow and migration scratch is exercised too): every batch's
    rows equal the oracle's; a plan refuses a second submit before its collect."""
    idx, q, _, oracle = setup
    plans = [idx.search_plan(128, (6, 1000, 150, 100)), idx.search_plan(128, (6, 1000, 150, 100))]
    rng = np.random.default_rng(9)
    batches = []
    for i in range(6):
        size = int(rng.integers(1, 129))
        rows = rng.choice(q.shape[0], size, replace=False)
        pick, params = _params(size, 100 + i)
        batches.append((rows, pick, params))
    pending = [None, None]
    for i, (rows, pick, params) in enumerate(batches):
        j = i % 2
        if pending[j] is not None:
            r0, p0 = pending[j]
            _check_rows(plans[j].collect(), p0, oracle(q[r0]))
        plans[j].submit(q[rows], params)
        if i == 0:
            with pytest.raises(efg.EfannaError):
                plans[0].submit(q[rows], params)
        pending[j] = (rows, pick)
    for j in (0, 1):
        r0, p0 = pending[j]
        _check_rows(plans[j].collect(), p0, oracle(q[r0]))
    for pl in plans:
        pl.close()


def test_batch_argument_errors(efg, setup):
    idx, q, _, _ = setup
    with pytest.raises(efg.EfannaError):
        idx.knn_search_batch(q[:2], [(4, 600, 100, 11), (4, 600, 100, 10)], 10)   # k above k_max
    with pytest.raises(efg.EfannaError):
        idx.knn_search_batch(q[:1], [(4, 0, 100, 1)], 10)                           # empty pool
    with pytest.raises(efg.EfannaError):
        idx.search_plan(16, (4, 10, 10, 20))                                         # k above pool


def test_seeded_search_matches_oracle(efg, oracle_lib, setup):
    """Entry seeds ahead of the tree leaves (ids >= n and repeats skipped) with per-query parameters."""
    O = oracle_lib
    idx, q, _, _ = setup
    g = load_golden("mid_d128")
    x = g["base"].astype(np.float32)
    forest = O.Forest.load(os.path.join(GOLDEN, "mid_d128.trees"))
    gp, gi = io.read_graph_csr(os.path.join(GOLDEN, "mid_d128.graph"))
    rng = np.random.default_rng(5)
    seeds = rng.integers(0, x.shape[0], (q.shape[0], 48)).astype(np.uint32)
    seeds[:, 7] = seeds[:, 3]                  # a repeat
    seeds[:, 11] = x.shape[0] + 5              # out of range
    pick, params = _params(q.shape[0], 7)
    params[:, 3] = np.minimum(params[:, 3], 10)
    ref = O.search_batch(x, forest, gp, gi, q, params, 10, trees=8, seeds=seeds, threads=4)
    Q = torch.from_numpy(q).cuda()
    P = torch.from_numpy(params).cuda()
    S = torch.from_numpy(seeds.view(np.int32)).cuda()
    out = torch.zeros((q.shape[0], 10), dtype=torch.int32, device="cuda")
    idx.knn_search_seeded_device(Q.data_ptr(), q.shape[0], q.shape[1], P.data_ptr(), (6, 1000, 150, 10),
                                 S.data_ptr(), 48, out.data_ptr())
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), ref)
    # pools made of seeds only (pool <= seeds per query)
    small = np.tile(np.array([2, 30, 30, 10], np.int32), (q.shape[0], 1))
    ref2 = O.search_batch(x, forest, gp, gi, q, small, 10, trees=8, seeds=seeds, threads=4)
    P2 = torch.from_numpy(small).cuda()
    idx.knn_search_seeded_device(Q.data_ptr(), q.shape[0], q.shape[1], P2.data_ptr(), (2, 30, 30, 10),
                                 S.data_ptr(), 48, out.data_ptr())
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), ref2)

