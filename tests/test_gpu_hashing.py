"""Hashing-seeded searches on the GPU (the reference's HASHINGIndex: pool/extend search,
algorithm/hashing_index.hpp:1087-1200, and kgraph search, :1203-1352): the probe sequence against a
plain-Python restatement of the reference's bucket visits, and both searches against the oracle's
canonical mode -- over the golden fixture's code sets (read back the way the reference reads its
code files) and larger Hamming balls."""
import itertools
import os

import numpy as np
import pytest
import torch

from conftest import GOLDEN, load_golden
from efanna_gb300 import datasets, io

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def case(efg):
    g = load_golden("small_d32")
    x, q = g["base"].astype(np.float32), g["queries"].astype(np.float32)
    idx = efg.Index(x, efg.IndexParams())
    idx.load_graph(os.path.join(GOLDEN, "small_d32.graph"))
    gp, gi = io.read_graph_csr(os.path.join(GOLDEN, "small_d32.graph"))
    hz = np.load(os.path.join(GOLDEN, "small_d32_hashing.npz"))
    yield idx, x, q, gp, gi, hz
    idx.close()


def probe_sequence(bcodes, qcodes, bits, radius, qi, cap):
    """The reference's visit order (getNeighborsIEH32_nnexp's loops): masks by radius, each radius's
    bit tuples in lexicographic order, tables inner, bucket members in id order; first cap entries."""
    seq = []
    buckets = []
    for t in range(bcodes.shape[0]):
        b = {}
        for i, c in enumerate(bcodes[t].tolist()):
            b.setdefault(c, []).append(i)
        buckets.append(b)
    for r in range(radius + 1):
        for tup in itertools.combinations(range(bits), r):
            m = sum(1 << p for p in tup)
            for t in range(bcodes.shape[0]):
                seq.extend(buckets[t].get(int(qcodes[t, qi]) ^ m, []))
                if len(seq) >= cap:
                    return seq[:cap]
    return seq + [0xFFFFFFFF] * (cap - len(seq))


def test_probe_sequence_matches_reference_order(efg, case):
    idx, x, q, gp, gi, hz = case
    for i in (0, 2, 4):
        clen, tables, up, rad, shift, ep, pool, ext, k = [int(v) for v in hz["points"][i]]
        bc, qc, bits = hz["bcodes_%d" % i].astype(np.uint64), hz["qcodes_%d" % i].astype(np.uint64), int(hz["bits_%d" % i])
        ht = efg.HashTables(idx, bc, bits, rad)
        assert ht.ball_size == sum(len(list(itertools.combinations(range(bits), r))) for r in range(rad + 1))
        cap = pool * tables
        QC = torch.from_numpy(qc.view(np.int64)).cuda()
        S = torch.zeros((q.shape[0], cap), dtype=torch.int32, device="cuda")
        ht.seeds_device(QC.data_ptr(), q.shape[0], q.shape[0], cap, S.data_ptr())
        torch.cuda.synchronize()
        got = S.cpu().numpy().view(np.uint32)
        for qi in range(0, q.shape[0], 7):
            assert got[qi].tolist() == probe_sequence(bc, qc, bits, rad, qi, cap), (i, qi)
        ht.close()


def test_search_matches_oracle_on_reference_code_sets(efg, oracle_lib, case):
    O = oracle_lib
    idx, x, q, gp, gi, hz = case
    for i, pt in enumerate(hz["points"]):
        clen, tables, up, rad, shift, ep, pool, ext, k = [int(v) for v in pt]
        bc, qc, bits = hz["bcodes_%d" % i].astype(np.uint64), hz["qcodes_%d" % i].astype(np.uint64), int(hz["bits_%d" % i])
        ht = efg.HashTables(idx, bc, bits, rad)
        idx.set_search_params(ep, pool, ext, 1, -1, 1)
        res = ht.search(k, q, qc)
        ref, _ = O.search_hashed(x, gp, gi, q, bc, qc, bits, rad, k=k, epochs=ep, init_num=pool, extend_to=ext,
                                 mode=O.CANON, threads=4)
        assert np.array_equal(res, ref), i
        # the device-pointer form gives the same rows
        Q = torch.from_numpy(q).cuda()
        QC = torch.from_numpy(qc.view(np.int64)).cuda()
        out = torch.zeros((q.shape[0], k), dtype=torch.int32, device="cuda")
        ht.search_device(Q.data_ptr(), q.shape[0], q.shape[1], QC.data_ptr(), q.shape[0], k, out.data_ptr())
        torch.cuda.synchronize()
        assert np.array_equal(out.cpu().numpy(), ref), i
        ht.close()


@pytest.mark.parametrize("bits,tables,radius,pool", [(40, 3, 3, 300), (64, 2, 2, 250), (24, 5, 2, 600), (8, 1, 8, 900)])
def test_search_matches_oracle_larger_balls(efg, oracle_lib, case, bits, tables, radius, pool):
    """Wide codes and deep radii (mask unranking up to bit 63, balls of thousands of masks), many
    tables, and a ball that covers every code (8 bits, radius 8)."""
    O = oracle_lib
    idx, x, q, gp, gi, _ = case
    bc = datasets.sign_codes(x, tables, bits, seed=bits)
    qc = datasets.sign_codes(q, tables, bits, seed=bits, center=x.mean(0))
    ht = efg.HashTables(idx, bc, bits, radius)
    idx.set_search_params(3, pool, 50, 1, -1, 1)
    res = ht.search(10, q, qc)
    ref, _ = O.search_hashed(x, gp, gi, q, bc, qc, bits, radius, k=10, epochs=3, init_num=pool, extend_to=50,
                             mode=O.CANON, threads=4)
    assert np.array_equal(res, ref)
    ht.close()


def test_kgraph_search_matches_oracle(efg, oracle_lib, case):
    """The hashing index's kgraph search (method 0 there): pools from the probe sequence, whole
    graph rows per expansion, the stored pool size raised to epochs * extend_to."""
    O = oracle_lib
    idx, x, q, gp, gi, hz = case
    for i, pt in enumerate(hz["points"]):
        clen, tables, up, rad, shift, ep, pool, ext, k = [int(v) for v in pt]
        bc, qc, bits = hz["bcodes_%d" % i].astype(np.uint64), hz["qcodes_%d" % i].astype(np.uint64), int(hz["bits_%d" % i])
        ht = efg.HashTables(idx, bc, bits, rad)
        idx.set_search_params(ep, pool, ext, 1, -1, 0)
        res = ht.search(k, q, qc)
        ref, _, _ = O.search_hashed_kgraph(x, gp, gi, q, bc, qc, bits, rad, k=k, epochs=ep, init_num=pool,
                                           extend_to=ext, mode=O.CANON, threads=4)
        assert np.array_equal(res, ref), i
        ht.close()
    # a 64-bit code set with a deeper ball
    bc = datasets.sign_codes(x, 2, 48, seed=9)
    qc = datasets.sign_codes(q, 2, 48, seed=9, center=x.mean(0))
    ht = efg.HashTables(idx, bc, 48, 2)
    idx.set_search_params(4, 300, 60, 1, -1, 0)
    ref, _, _ = O.search_hashed_kgraph(x, gp, gi, q, bc, qc, 48, 2, k=10, epochs=4, init_num=300, extend_to=60,
                                       mode=O.CANON, threads=4)
    assert np.array_equal(ht.search(10, q, qc), ref)
    ht.close()


def test_bucket_search_without_graph_matches_oracle(efg, oracle_lib, case):
    """The hashing index without a graph (getNeighbors32 / _64): bucket ids ranked, the random fill
    only up to k."""
    O = oracle_lib
    _, x, q, _, _, hz = case
    idx = efg.Index(x, efg.IndexParams())
    for i, pt in enumerate(hz["points"]):
        clen, tables, up, rad, shift, ep, pool, ext, k = [int(v) for v in pt]
        bc, qc, bits = hz["bcodes_%d" % i].astype(np.uint64), hz["qcodes_%d" % i].astype(np.uint64), int(hz["bits_%d" % i])
        ht = efg.HashTables(idx, bc, bits, rad)
        idx.set_search_params(ep, pool, ext, 1, -1, 1)
        ref = O.search_hashed_buckets(x, q, bc, qc, bits, rad, k=k, init_num=pool, mode=O.CANON, threads=4)
        assert np.array_equal(ht.search(k, q, qc), ref), i
        ht.close()
    idx.close()


def test_hash_argument_errors(efg, case):
    idx, x, q, *_ = case
    bc = datasets.sign_codes(x, 2, 16, seed=1)
    with pytest.raises(efg.EfannaError):
        efg.HashTables(idx, bc, 16, 17)          # radius above the code length
    with pytest.raises(efg.EfannaError):
        efg.HashTables(idx, bc, 12, 1)           # codes wider than code_bits
    with pytest.raises(efg.EfannaError):
        efg.HashTables(idx, datasets.sign_codes(x, 2, 64, seed=1), 64, 6)  # ball of ~7.6e7 masks x 2 tables
    ht = efg.HashTables(idx, bc, 16, 1)
    idx.set_search_params(3, 200, 40, 1, -1, 1)
    with pytest.raises(efg.EfannaError):
        ht.search(201, q, datasets.sign_codes(q, 2, 16, seed=1))  # k above the pool
    assert ht.search(10, q[:0], np.zeros((2, 0), np.uint64)).shape == (0, 10)
    ht.close()


def test_reference_api_program_through_facade(efg, oracle_lib, case, tmp_path):
    """A program written against the reference's API (HASHINGIndexParams, FIndex::buildIndex,
    loadGraph, setSearchParams(..., 1), knnSearch, saveResults), compiled against the facade: its
    results file equals the oracle's canonical search."""
    import subprocess
    from test_dropin import build_hashing_driver
    O = oracle_lib
    idx, x, q, gp, gi, hz = case
    exe = build_hashing_driver(efg, tmp_path)
    bf, qf, rf = str(tmp_path / "b.fvecs"), str(tmp_path / "q.fvecs"), str(tmp_path / "r.ivecs")
    io.write_fvecs(bf, x)
    io.write_fvecs(qf, q)
    for i, method in ((0, 1), (1, 1), (2, 1), (0, 0), (2, 0), (0, -1), (3, -1)):  # -1: no graph
        clen, tables, up, rad, shift, ep, pool, ext, k = [int(v) for v in hz["points"][i]]
        bc, qc, bits = hz["bcodes_%d" % i].astype(np.uint64), hz["qcodes_%d" % i].astype(np.uint64), int(hz["bits_%d" % i])
        # the files hold the codes before the shift (any low bits: the reader drops them)
        io.write_codes(str(tmp_path / "bc"), bc << np.uint64(shift), clen)
        io.write_codes(str(tmp_path / "qc"), qc << np.uint64(shift), clen)
        graph = os.path.join(GOLDEN, "small_d32.graph") if method >= 0 else "-"
        r = subprocess.run([exe, bf, graph, qf, str(tmp_path / "bc"), str(tmp_path / "qc"), rf, str(clen), str(tables),
                            str(up), str(rad), str(shift), str(ep), str(pool), str(ext), str(k), str(method if method >= 0 else 1)],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stdout + r.stderr
        if method < 0:
            ref = O.search_hashed_buckets(x, q, bc, qc, bits, rad, k=k, init_num=pool, mode=O.CANON, threads=4)
        elif method == 1:
            ref, _ = O.search_hashed(x, gp, gi, q, bc, qc, bits, rad, k=k, epochs=ep, init_num=pool, extend_to=ext,
                                     mode=O.CANON, threads=4)
        else:
            ref, _, _ = O.search_hashed_kgraph(x, gp, gi, q, bc, qc, bits, rad, k=k, epochs=ep, init_num=pool,
                                               extend_to=ext, mode=O.CANON, threads=4)
        assert np.array_equal(io.read_ivecs(rf), ref), (i, method)
        # outputVisitBucketNum after the search prints the reference's histogram lines
        key = {1: "visit_%d", 0: "visit_kgraph_%d", -1: "visit_buckets_%d"}[method] % i
        lines = [ln for ln in r.stdout.splitlines() if ln.startswith("Radius")]
        assert lines == [str(v) for v in hz[key]], (i, method, lines)
