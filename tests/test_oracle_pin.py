"""The CPU oracle against the reference's own outputs (golden fixtures made by
tests/golden/make_golden.py from the reference compiled here, single-threaded)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, load_golden
from efanna_gb300 import io

CASES = ["small_d32", "mid_d128"]


def _params(O, gp):
    trees, ml, ep, L, ck, K, S = [int(v) for v in gp]
    return O.make_params(K=K, S=S, L=L, check_k=ck, epochs=ep, trees=trees, merge_level=ml)


@pytest.mark.parametrize("case", CASES)
def test_seq_graph_matches_reference_bytes(oracle_lib, case):
    O = oracle_lib
    g = load_golden(case)
    x = g["base"].astype(np.float32)
    rc, gs, forest, _ = O.build_graph(x, _params(O, g["graph_params"]), O.SEQ)
    assert rc == 0
    ref = np.fromfile(os.path.join(GOLDEN, case + ".graph"), np.uint32).reshape(x.shape[0], -1)
    assert np.all(ref[:, 0] == gs.shape[1])
    assert np.array_equal(ref[:, 1:], gs)


def _tree_records(path):
    """Trees file with the raw child-pointer words reduced to null / non-null."""
    import struct
    A = bytearray(open(path, "rb").read())
    K, T, N, D = struct.unpack_from("<IIQQ", A, 0)
    off = 24
    for _ in range(T):
        nn, _ns = struct.unpack_from("<ii", A, off)
        off += 8
        for _ in range(nn):
            lp, rp = struct.unpack_from("<QQ", A, off + 24)
            struct.pack_into("<QQ", A, off + 24, int(lp != 0), int(rp != 0))
            off += 40
    return bytes(A)


@pytest.mark.parametrize("case", CASES)
def test_seq_trees_match_reference_bytes(oracle_lib, case, tmp_path):
    O = oracle_lib
    g = load_golden(case)
    x = g["base"].astype(np.float32)
    rc, gs, forest, _ = O.build_graph(x, _params(O, g["graph_params"]), O.SEQ)
    out = str(tmp_path / "o.trees")
    forest.save(out, int(g["graph_params"][5]))
    assert _tree_records(out) == _tree_records(os.path.join(GOLDEN, case + ".trees"))


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("mode", ["seq", "canon", "omp"])
def test_search_matches_reference_results(oracle_lib, case, mode):
    """SEQ and OMP (the timed reference arm's search, queries spread over threads) give the
    reference's result ids byte for byte; so does CANON on these fixtures."""
    O = oracle_lib
    g = load_golden(case)
    x = g["base"].astype(np.float32)
    q = g["queries"].astype(np.float32)
    st, se, pool, ext, k = [int(v) for v in g["search_params"]]
    forest = O.Forest.load(os.path.join(GOLDEN, case + ".trees"))
    gp, gi = io.read_graph_csr(os.path.join(GOLDEN, case + ".graph"))
    out = O.search(x, forest, gp, gi, q, k=k, epochs=se, init_num=pool, extend_to=ext, trees=st,
                   mode={"seq": O.SEQ, "canon": O.CANON, "omp": O.OMP}[mode], threads=1 if mode == "seq" else 4)
    assert np.array_equal(out, g["results"])


def test_merge_level_error_matches_reference(oracle_lib):
    """The reference aborts with 'merge level deeper than tree, max merge deepth is 5' on this case."""
    O = oracle_lib
    g = load_golden("small_d32")
    x = g["base"].astype(np.float32)
    rc, gs, forest, maxd = O.build_graph(x, O.make_params(merge_level=8), O.SEQ)
    assert rc == 3 and maxd == 5
    rc, gs, forest, maxd = O.build_graph(x, O.make_params(merge_level=8), O.CANON)
    assert rc == 3


def _exact_knn_u8(x, rows, k=10):
    """Exact k-NN (self excluded) of base rows `rows` by the Gram form in FP32: on integer data in
    [0, 255] with d <= 128 every partial sum is an integer below 2^24, so the distances are exact."""
    xf = x.astype(np.float32)
    sq = (xf * xf).sum(1)
    out = np.zeros((len(rows), k), np.int64)
    for b in range(0, len(rows), 2000):
        r = rows[b:b + 2000]
        D = sq[r][:, None] + sq[None, :] - 2 * (xf[r] @ xf.T)
        D[np.arange(len(r)), r] = np.inf
        part = np.argpartition(D, k, axis=1)[:, :k]
        out[b:b + len(r)] = part
    return out


def _graph_recall(gs, gt, rows):
    return float(np.mean([len(set(gs[r][:10].tolist()) & set(gt[i].tolist())) for i, r in enumerate(rows)]) / 10)


def test_canonical_recall_equivalent(oracle_lib):
    """The order-independent restatement reaches the reference order's graph quality: mean
    |recall@10(SEQ) - recall@10(CANON)| over three seeded data sets within 0.005, the parity window
    for graph recall against the reference."""
    O = oracle_lib
    from efanna_gb300 import datasets
    p = O.make_params(merge_level=5, epochs=6)
    diffs = []
    for seed in (3, 4, 5):
        x = datasets.mixture_u8(6000, 64, seed=seed)
        rows = np.arange(len(x))
        gt = _exact_knn_u8(x, rows)
        rec = {}
        for mode in (O.SEQ, O.CANON):
            rc, gs, _, _ = O.build_graph(x, p, mode)
            assert rc == 0
            rec[mode] = _graph_recall(gs, gt, rows)
        print("seed", seed, "SEQ %.5f CANON %.5f" % (rec[O.SEQ], rec[O.CANON]))
        diffs.append(rec[O.SEQ] - rec[O.CANON])
    assert abs(np.mean(diffs)) <= 0.005, diffs
    assert max(abs(d) for d in diffs) <= 0.01, diffs


def _ref_recall_100k():
    import json
    ref = json.load(open(os.path.join(GOLDEN, "ref_recall_100k.json")))
    multi = [r["recall_at_10"] for r in ref["runs"] if r["threads"] > 1]
    return ref, multi


def test_omp_graph_recall_matches_reference_at_100k(oracle_lib):
    """The timed reference arm's build (the OpenMP restatement) against the reference's own
    multi-threaded builds at N = 100,000 x 128 with (trees, ml, iter, L, check, K, S) = (8, 8, 8,
    30, 25, 10, 10) (tests/golden/ref_recall_100k.json, recorded by make_golden.py): its graph
    recall@10 on 5,000 sampled rows lies within 0.005 of their mean."""
    O = oracle_lib
    from efanna_gb300 import datasets
    ref, multi = _ref_recall_100k()
    x = datasets.mixture_u8(100000, 128, seed=0)
    p = O.make_params(K=10, S=10, L=30, check_k=25, epochs=8, trees=8, merge_level=8)
    rc, gs, _, _ = O.build_graph(x, p, O.OMP)
    assert rc == 0
    rows = np.sort(np.random.default_rng(11).choice(len(x), 5000, replace=False))
    rec = _graph_recall(gs, _exact_knn_u8(x, rows), rows)
    print("OMP restatement %.5f, reference runs %s (mean %.5f)" % (rec, multi, np.mean(multi)))
    assert abs(rec - np.mean(multi)) <= 0.005


def test_l2_orders_agree_on_integers(oracle_lib):
    O = oracle_lib
    rng = np.random.default_rng(0)
    for d in (8, 32, 128, 96, 960):
        a = rng.integers(0, 256, d).astype(np.float32)
        b = rng.integers(0, 256, d).astype(np.float32)
        exact = float(((a.astype(np.int64) - b.astype(np.int64)) ** 2).sum())
        assert O.l2(a, b, "avx") == exact
        assert O.l2(a, b, "scalar") == exact


def test_l2_avx_tail_quirk(oracle_lib):
    """L2DistanceAVX sums only 8 of the 16/24 padded tail floats (distance.hpp:305-314)."""
    O = oracle_lib
    d = 48  # D % 32 == 16
    a = np.ones(d, np.float32)
    b = np.zeros(d, np.float32)
    assert O.l2(a, b, "scalar") == 48.0
    assert O.l2(a, b, "avx") == 40.0


def _kgraph_case(O, case):
    g = load_golden(case)
    kg = np.load(os.path.join(GOLDEN, case + "_kgraph.npz"))
    forest = O.Forest.load(os.path.join(GOLDEN, case + ".trees"))
    gp, gi = io.read_graph_csr(os.path.join(GOLDEN, case + ".graph"))
    return g["base"].astype(np.float32), g["queries"].astype(np.float32), kg, forest, gp, gi


@pytest.mark.parametrize("case", CASES)
def test_kgraph_seq_matches_reference_results(oracle_lib, case):
    """getNeighbors_kgraph restated: byte-identical ids to the reference's own search method 1,
    including a second call on the enlarged pool size."""
    O = oracle_lib
    x, q, kg, forest, gp, gi = _kgraph_case(O, case)
    for i, (st, ep, pool, ext, k) in enumerate(kg["points"]):
        out, _, pool2 = O.search_kgraph(x, forest, gp, gi, q, k=int(k), epochs=int(ep), init_num=int(pool),
                                        extend_to=int(ext), trees=int(st), mode=O.SEQ)
        assert np.array_equal(out, kg["first_%d" % i]), (case, i)
        assert pool2 == (max(int(pool), int(ep) * int(ext)))
        out2, _, _ = O.search_kgraph(x, forest, gp, gi, q, k=int(k), epochs=int(ep), init_num=pool2,
                                     extend_to=int(ext), trees=int(st), mode=O.SEQ)
        assert np.array_equal(out2, kg["second_%d" % i]), (case, i)


@pytest.mark.parametrize("case", CASES)
def test_kgraph_canonical_close_to_reference(oracle_lib, case):
    """The canonical restatement orders equal distances by id instead of by arrival; on the
    integer-valued fixtures that moves at most a few ids per thousand, never the recall."""
    O = oracle_lib
    x, q, kg, forest, gp, gi = _kgraph_case(O, case)
    for i, (st, ep, pool, ext, k) in enumerate(kg["points"]):
        out, _, _ = O.search_kgraph(x, forest, gp, gi, q, k=int(k), epochs=int(ep), init_num=int(pool),
                                    extend_to=int(ext), trees=int(st), mode=O.CANON, threads=4)
        ref = kg["first_%d" % i]
        assert np.mean(out == ref) > 0.99
        same_sets = np.mean([len(set(a) & set(b)) / len(a) for a, b in zip(out, ref)])
        assert same_sets > 0.995


def _hashing_case():
    g = load_golden("small_d32")
    hz = np.load(os.path.join(GOLDEN, "small_d32_hashing.npz"))
    gp, gi = io.read_graph_csr(os.path.join(GOLDEN, "small_d32.graph"))
    return g["base"].astype(np.float32), g["queries"].astype(np.float32), hz, gp, gi


def test_hashing_seq_matches_reference_results(oracle_lib):
    """getNeighborsIEH32_nnexp / IEH64_nnexp restated: byte-identical ids to the reference's
    hashing initialiser (search method 1 there) for 32- and 64-bit code files, a code shift, pools
    filled from the buckets and pools topped up by the random fill."""
    O = oracle_lib
    x, q, hz, gp, gi = _hashing_case()
    for i, (clen, tables, up, rad, shift, ep, pool, ext, k) in enumerate(hz["points"]):
        out, _ = O.search_hashed(x, gp, gi, q, hz["bcodes_%d" % i], hz["qcodes_%d" % i], int(hz["bits_%d" % i]),
                                 int(rad), k=int(k), epochs=int(ep), init_num=int(pool), extend_to=int(ext),
                                 mode=O.SEQ)
        assert np.array_equal(out, hz["results_%d" % i]), i


def test_hashing_canonical_close_to_reference(oracle_lib):
    """The canonical mode's random fill and tie order differ from std::rand() and arrival order.
    Where the buckets fill the pool the results agree almost everywhere; point 1 (40-bit codes at
    radius 1 over 3000 points) hits few buckets, so its pool is mostly random fill and only its
    recall is comparable."""
    O = oracle_lib
    x, q, hz, gp, gi = _hashing_case()
    d = (q * q).sum(1)[:, None] + (x * x).sum(1)[None, :] - 2 * q.astype(np.float64) @ x.T.astype(np.float64)
    gt = np.argsort(d, 1, kind="stable")[:, :10]

    def recall(r):
        return np.mean([len(set(a[:10]) & set(b)) / 10 for a, b in zip(r, gt)])

    for i, (clen, tables, up, rad, shift, ep, pool, ext, k) in enumerate(hz["points"]):
        out, _ = O.search_hashed(x, gp, gi, q, hz["bcodes_%d" % i], hz["qcodes_%d" % i], int(hz["bits_%d" % i]),
                                 int(rad), k=int(k), epochs=int(ep), init_num=int(pool), extend_to=int(ext),
                                 mode=O.CANON, threads=4)
        ref = hz["results_%d" % i]
        same_sets = np.mean([len(set(a) & set(b)) / len(a) for a, b in zip(out, ref)])
        assert abs(recall(out) - recall(ref)) < 0.03, i
        if i != 1:
            assert same_sets > 0.97, (i, same_sets)


def test_hashing_kgraph_seq_matches_reference_results(oracle_lib):
    """getNeighborsIEH32_kgraph / IEH64_kgraph restated (whole graph rows per expansion, the pool
    size raised to epochs * extend_to where that is not smaller): byte-identical ids to the
    reference's hashing kgraph search (search method 0 there)."""
    O = oracle_lib
    x, q, hz, gp, gi = _hashing_case()
    for i, (clen, tables, up, rad, shift, ep, pool, ext, k) in enumerate(hz["points"]):
        out, _, pool2 = O.search_hashed_kgraph(x, gp, gi, q, hz["bcodes_%d" % i], hz["qcodes_%d" % i],
                                               int(hz["bits_%d" % i]), int(rad), k=int(k), epochs=int(ep),
                                               init_num=int(pool), extend_to=int(ext), mode=O.SEQ)
        assert np.array_equal(out, hz["kgraph_%d" % i]), i
        assert pool2 == max(int(pool), int(ep) * min(int(ext), int(pool)))


def test_hashing_bucket_search_seq_matches_reference_results(oracle_lib):
    """getNeighbors32 / getNeighbors64 restated (the hashing index without a graph: bucket ids,
    random fill to k only, ranked): byte-identical ids to the reference's."""
    O = oracle_lib
    x, q, hz, gp, gi = _hashing_case()
    for i, (clen, tables, up, rad, shift, ep, pool, ext, k) in enumerate(hz["points"]):
        out = O.search_hashed_buckets(x, q, hz["bcodes_%d" % i], hz["qcodes_%d" % i], int(hz["bits_%d" % i]),
                                      int(rad), k=int(k), init_num=int(pool), mode=O.SEQ)
        assert np.array_equal(out, hz["buckets_%d" % i]), i
