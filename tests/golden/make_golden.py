"""Regenerates the golden fixtures in this folder from the reference's own programs.

Run here (where the reference sources are) with ``python tests/golden/make_golden.py``.  It
compiles the reference samples with oracle/Makefile, runs them single-threaded (byte-identical
across runs) on small seeded integer-valued data, and stores inputs and outputs:

  <case>.npz   base (uint8), queries (uint8), search parameters, the reference's search results,
               the reference's graph rows, and the params used to build them
  <case>.trees the reference's trees file (buildall), byte-for-byte
  <case>.graph the reference's graph file, byte-for-byte
  ref_recall_100k.json  graph recall@10 of the reference's multi-threaded build at N=100k (3 runs
               + 1 single-thread run) against exact 10-NN, with build times on this host.
  <case>_kgraph.npz  the reference's kgraph search (search method 1, through its FIndex API via
               oracle/ref_drivers/kgraph_search.cc) on the case's trees and graph files, for each
               parameter set in KGRAPH_POINTS: the first call's ids and a second call's ids on the
               same index (the first call may enlarge the stored pool size).

  <case>_hashing.npz  the reference's hashing-seeded search (HASHINGIndex, search method 1, through
               its FIndex API via oracle/ref_drivers/hashing_search.cc) on the case's graph file with
               seeded sign-of-projection codes (datasets.sign_codes) written as the reference's code
               files, for each parameter set in HASH_POINTS: the codes as read back (tables x n and
               tables x nq, after the shift), the code length in effect and the ids; the same for
               its kgraph search (search method 0 there) as kgraph_<i> and for its search without
               a graph (the bucket search) as buckets_<i>; the lines outputVisitBucketNum printed
               after each search as visit_<i>, visit_kgraph_<i>, visit_buckets_<i>.

``--only-kgraph`` / ``--only-hashing`` regenerate just those fixtures.

The data are stored (as uint8) rather than regenerated so that the fixtures do not depend on the
platform's numpy.
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402
from efanna_gb300 import datasets, io  # noqa: E402

CASES = {
    # name: (n, d, nq, graph params (trees, ml, epochs, L, check, K, S), search (trees, epochs, pool, extend, k))
    "small_d32": (3000, 32, 200, (8, 4, 8, 30, 25, 10, 10), (8, 4, 400, 50, 10)),
    "mid_d128": (4000, 128, 200, (8, 5, 6, 30, 25, 10, 10), (8, 4, 600, 100, 10)),
}


# kgraph search points (trees, epochs, pool, extend, k): sorted pools (epochs * extend < pool) and
# pools the reference enlarges to epochs * extend.
KGRAPH_POINTS = [(8, 4, 400, 50, 10), (8, 4, 100, 50, 10), (8, 3, 600, 40, 20), (4, 2, 150, 100, 10),
                 (8, 5, 200, 30, 5)]


# hashing search points (code length, tables, upper bits, radius, shift, epochs, pool, extend, k):
# 32- and 64-bit code files, a shift, pools filled from the buckets and pools the random fill tops up.
HASH_POINTS = [(12, 2, 4, 2, 0, 4, 200, 40, 10), (40, 3, 8, 1, 0, 3, 150, 30, 10), (16, 2, 5, 3, 2, 2, 300, 300, 20),
               (10, 1, 3, 2, 0, 4, 2500, 50, 10), (20, 4, 6, 1, 0, 4, 400, 60, 10)]


def run(cmd, threads):
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    r = subprocess.run(cmd, env=env, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(" ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout


def make_case(name, n, d, nq, gp, sp, tmp):
    x = datasets.mixture_u8(n, d, seed=0)
    q = datasets.mixture_u8(nq, d, seed=0, queries=True)
    base, qf = os.path.join(tmp, "b.fvecs"), os.path.join(tmp, "q.fvecs")
    io.write_fvecs(base, x)
    io.write_fvecs(qf, q)
    g, t, r = os.path.join(HERE, name + ".graph"), os.path.join(HERE, name + ".trees"), os.path.join(tmp, "r.ivecs")
    trees, ml, ep, L, ck, K, S = gp
    run([O.ref_bin("efanna_index_buildall", "strict"), base, g, t, str(trees), str(ml), str(ep), str(L), str(ck),
         str(K), str(S)], 1)
    st, se, pool, ext, k = sp
    run([O.ref_bin("efanna_search", "strict"), base, t, g, qf, r, str(st), str(se), str(pool), str(ext), str(k)], 1)
    res = io.read_ivecs(r)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), base=x.astype(np.uint8), queries=q.astype(np.uint8),
                        graph_params=np.array(gp), search_params=np.array(sp), results=res)


def make_kgraph(name, tmp):
    g = np.load(os.path.join(HERE, name + ".npz"))
    base, qf, r = os.path.join(tmp, "b.fvecs"), os.path.join(tmp, "q.fvecs"), os.path.join(tmp, "r.ivecs")
    io.write_fvecs(base, g["base"].astype(np.float32))
    io.write_fvecs(qf, g["queries"].astype(np.float32))
    first, second = [], []
    for st, ep, pool, ext, k in KGRAPH_POINTS:
        run([O.ref_bin("kgraph_search", "strict"), base, os.path.join(HERE, name + ".trees"),
             os.path.join(HERE, name + ".graph"), qf, r, str(st), str(ep), str(pool), str(ext), str(k), "2"], 1)
        first.append(io.read_ivecs(r))
        second.append(io.read_ivecs(r + ".2"))
    np.savez_compressed(os.path.join(HERE, name + "_kgraph.npz"), points=np.array(KGRAPH_POINTS),
                        **{"first_%d" % i: a for i, a in enumerate(first)},
                        **{"second_%d" % i: a for i, a in enumerate(second)})


def make_hashing(name, tmp):
    g = np.load(os.path.join(HERE, name + ".npz"))
    x, q = g["base"].astype(np.float32), g["queries"].astype(np.float32)
    base, qf, r = os.path.join(tmp, "b.fvecs"), os.path.join(tmp, "q.fvecs"), os.path.join(tmp, "r.ivecs")
    io.write_fvecs(base, x)
    io.write_fvecs(qf, q)
    bpre, qpre = os.path.join(tmp, "bc"), os.path.join(tmp, "qc")
    out = {"points": np.array(HASH_POINTS)}
    for i, (clen, tables, up, rad, shift, ep, pool, ext, k) in enumerate(HASH_POINTS):
        io.write_codes(bpre, datasets.sign_codes(x, tables, clen, seed=100 + i), clen)
        io.write_codes(qpre, datasets.sign_codes(q, tables, clen, seed=100 + i, center=x.mean(0)), clen)
        args = [O.ref_bin("hashing_search", "strict"), base, os.path.join(HERE, name + ".graph"), qf, bpre, qpre, r,
                str(clen), str(tables), str(up), str(rad), str(shift), str(ep), str(pool), str(ext), str(k)]
        def radius_lines(text):
            return np.array([ln for ln in text.splitlines() if ln.startswith("Radius")])

        out["visit_kgraph_%d" % i] = radius_lines(run(args + ["0"], 1))
        out["kgraph_%d" % i] = io.read_ivecs(r)
        out["visit_buckets_%d" % i] = radius_lines(run(args[:2] + ["-"] + args[3:], 1))
        out["buckets_%d" % i] = io.read_ivecs(r)
        out["visit_%d" % i] = radius_lines(run(args, 1))
        bc, bits = io.read_codes(bpre, tables, clen, shift)
        qc, _ = io.read_codes(qpre, tables, clen, shift)
        word = np.uint32 if bits <= 32 else np.uint64
        out.update({"bcodes_%d" % i: bc.astype(word), "qcodes_%d" % i: qc.astype(word), "bits_%d" % i: bits,
                    "results_%d" % i: io.read_ivecs(r)})
    np.savez_compressed(os.path.join(HERE, name + "_hashing.npz"), **out)


def exact_knn(x, k):
    xd = x.astype(np.float64)
    nrm = (xd * xd).sum(1)
    out = np.zeros((x.shape[0], k), np.int64)
    for s in range(0, x.shape[0], 2000):
        D = nrm[s:s + 2000, None] + nrm[None, :] - 2 * xd[s:s + 2000] @ xd.T
        D[np.arange(D.shape[0]), np.arange(s, s + D.shape[0])] = np.inf
        part = np.argpartition(D, k, axis=1)[:, :k]
        dd = np.take_along_axis(D, part, 1)
        out[s:s + 2000] = np.take_along_axis(part, np.lexsort((part, dd), axis=1), 1)
    return out


def ref_recall_100k(tmp):
    n, d = 100_000, 128
    x = datasets.mixture_u8(n, d, seed=0)
    base = os.path.join(tmp, "b100k.fvecs")
    io.write_fvecs(base, x)
    gt = exact_knn(x, 10)
    runs = []
    for threads in (0, 0, 0, 1):
        g = os.path.join(tmp, "g100k.graph")
        t0 = time.time()
        cmd = [O.ref_bin("efanna_index_buildgraph", "stock"), base, g, "8", "8", "8", "30", "25", "10", "10"]
        run(cmd, threads or os.cpu_count())
        wall = time.time() - t0
        gs = np.fromfile(g, np.uint32).reshape(n, 11)[:, 1:]
        rec = float(np.mean([len(set(gs[i]) & set(gt[i])) for i in range(n)]) / 10)
        runs.append({"threads": threads or os.cpu_count(), "recall_at_10": rec, "wall_s": wall})
    json.dump({"n": n, "d": d, "params": "trees=8 ml=8 iter=8 L=30 check=25 K=10 S=10",
               "generator": "datasets.mixture_u8(100000, 128, seed=0)", "host_cpus": os.cpu_count(),
               "runs": runs}, open(os.path.join(HERE, "ref_recall_100k.json"), "w"), indent=1)


if __name__ == "__main__":
    O.build()
    if not O.build_ref():
        sys.exit("reference sources not found; fixtures unchanged")
    only = [a for a in sys.argv if a.startswith("--only-")]
    with tempfile.TemporaryDirectory() as tmp:
        if not only:
            for name, spec in CASES.items():
                make_case(name, *spec, tmp)
        if not only or "--only-kgraph" in only:
            for name in CASES:
                make_kgraph(name, tmp)
        if not only or "--only-hashing" in only:
            make_hashing("small_d32", tmp)
        if "--skip-100k" not in sys.argv and not only:
            ref_recall_100k(tmp)
