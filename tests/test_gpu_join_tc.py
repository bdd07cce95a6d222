"""The NN-descent join on the tensor cores (efg_set_build_precision 'bf16') against the oracle and
the FP32 join.

On byte-valued data up to 128 dimensions every Gram value, norm and distance is an integer below
2^24, so the tensor-core join must leave exactly the oracle's state after every iteration (the FP32
join's is pinned to it by test_gpu_parity) and build the identical graph.  Nodes too large for one
tile (more than 128 new entries or 256 rows) are scored tile by tile in a second launch; one case
here has many.  On
real-valued data (hi + lo products) the graph may differ where distances tie within the split's
error; its recall against exact neighbours must stay within 0.005 of the FP32 build's.
"""
import numpy as np
import pytest

from efanna_gb300 import datasets

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _state_diff(a, b):
    for f in a.FIELDS:
        va, vb = getattr(a, f), getattr(b, f)
        if f in ("new_ids", "old_ids"):
            cnt = a.new_cnt if f == "new_ids" else a.old_cnt
            for i in range(a.n):
                if not np.array_equal(va[i, :cnt[i]], vb[i, :cnt[i]]):
                    return "%s row %d" % (f, i)
        elif not np.array_equal(va, vb):
            return "%s row %d" % (f, int(np.argwhere(va != vb)[0][0]))
    return None


STATE_CASES = [
    (3000, 32, dict(trees=8, merge_level=4, epochs=4, check=25, L=30, K=10, S=10)),
    (2500, 128, dict(trees=4, merge_level=3, epochs=3, check=40, L=20, K=8, S=6)),
    (2000, 64, dict(trees=6, merge_level=4, epochs=3, check=60, L=50, K=20, S=12)),
    (1500, 96, dict(trees=4, merge_level=3, epochs=3, check=150, L=150, K=20, S=10)),
]


@pytest.mark.parametrize("n,d,params", STATE_CASES)
def test_tc_join_iterations_match_oracle(efg, oracle_lib, n, d, params):
    O = oracle_lib
    x = datasets.mixture_u8(n, d, seed=11)
    p = O.make_params(K=params["K"], S=params["S"], L=params["L"], check_k=params["check"],
                      epochs=params["epochs"], trees=params["trees"], merge_level=params["merge_level"])
    forest = O.Forest.build(x, params["trees"], S=params["S"], mode=O.CANON)
    cap = max(p.L, 2 * p.S) + p.reverse_cap
    rc, st = O.nnd_init(x, forest, p, cap, O.CANON)
    assert rc == 0
    idx = efg.Index(x, efg.IndexParams(**params))
    idx.set_build_precision("bf16")
    cur = st
    for it in range(params["epochs"]):
        nxt, pairs = O.nnd_iterate(x, cur, p, it, O.CANON)
        g = cur.copy()
        assert idx.nnd_iterate(g, it) == pairs
        assert _state_diff(nxt, g) is None, (it, _state_diff(nxt, g))
        cur = nxt


def test_tc_join_oversized_lists_match_oracle(efg, oracle_lib):
    """Nodes beyond one tile (more than 128 new entries, or more than 256 rows) are scored as
    blocks of new entries x chunks of candidates; lists that large do not arise at test sizes, so
    some nodes of a real initial state get long random lists (any lists are a valid join input)."""
    O = oracle_lib
    n, d = 3000, 32
    params = dict(trees=4, merge_level=3, epochs=1, check=40, L=30, K=10, S=10, reverse_cap=400)
    x = datasets.mixture_u8(n, d, seed=13)
    p = O.make_params(K=10, S=10, L=30, check_k=40, epochs=1, trees=4, merge_level=3, reverse_cap=400)
    forest = O.Forest.build(x, 4, S=10, mode=O.CANON)
    cap = max(p.L, 2 * p.S) + p.reverse_cap
    rc, st = O.nnd_init(x, forest, p, cap, O.CANON)
    assert rc == 0
    rng = np.random.default_rng(5)
    sizes = [(140, 100), (129, 0), (100, 200), (20, 237), (128, 128), (1, 300), (60, 150)]
    for j, i in enumerate(rng.choice(n, 70, replace=False)):
        nn, no = sizes[j % len(sizes)]
        ids = rng.choice(np.delete(np.arange(n), i), nn + no, replace=False).astype(st.new_ids.dtype)
        st.new_ids[i, :nn], st.new_cnt[i] = ids[:nn], nn
        st.old_ids[i, :no], st.old_cnt[i] = ids[nn:], no
    nn, no = st.new_cnt.astype(np.int64), st.old_cnt.astype(np.int64)
    big = int(((nn > 128) | (nn + no > 256)).sum())
    assert big >= 40
    idx = efg.Index(x, efg.IndexParams(**params))
    idx.set_build_precision("bf16")
    nxt, pairs = O.nnd_iterate(x, st, p, 0, O.CANON)
    g = st.copy()
    assert idx.nnd_iterate(g, 0) == pairs
    assert _state_diff(nxt, g) is None, _state_diff(nxt, g)


def _build(efg, x, precision, **params):
    idx = efg.Index(x, efg.IndexParams(**params))
    idx.set_build_precision(precision)
    idx.build_index()
    return idx


@pytest.mark.parametrize("d", [128, 100, 7])
def test_tc_join_graph_identical_on_byte_data(efg, d):
    x = datasets.mixture_u8(30000, d, seed=5).astype(np.float32)
    params = dict(trees=8, merge_level=5, epochs=6, check=25, L=30, K=10, S=10)
    a = _build(efg, x, "fp32", **params)
    b = _build(efg, x, "bf16", **params)
    assert np.array_equal(a.graph(), b.graph())
    sa, sb = a.build_stats(), b.build_stats()
    assert sa.join_pairs == sb.join_pairs and sa.join_records == sb.join_records
    assert sa.join_large_nodes == 0 and sb.join_large_nodes == 0


def test_tc_join_float_data_recall(efg):
    n, d, k = 40000, 96, 10
    x = datasets.mixture_unit(n, d, seed=4)
    params = dict(trees=8, merge_level=5, epochs=6, check=25, L=30, K=k, S=10)
    X = torch.from_numpy(x).cuda()
    gt = torch.empty((n, k), dtype=torch.int32, device="cuda")
    efg.brute_force_knn_device(X.data_ptr(), n, d, d, X.data_ptr(), n, d, k, gt.data_ptr(), exclude_self=True)
    gt = gt.cpu().numpy()

    def recall(g):
        return np.mean([len(set(r[:k]) & set(t)) / k for r, t in zip(g, gt)])

    r32 = recall(_build(efg, x, "fp32", **params).graph())
    r16 = recall(_build(efg, x, "bf16", **params).graph())
    assert r16 >= r32 - 0.005, (r16, r32)


def test_build_precision_argument_errors(efg):
    x = datasets.mixture_u8(500, 8, seed=1).astype(np.float32)
    idx = efg.Index(x, efg.IndexParams(trees=2, merge_level=2, epochs=1, check=10, L=10, K=5, S=5))
    with pytest.raises(ValueError):
        idx.set_build_precision("fp8")
    with pytest.raises(efg.EfannaError):
        efg._check(efg.lib().efg_set_build_precision(idx._h, 2))
