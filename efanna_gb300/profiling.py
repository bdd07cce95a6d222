"""Profiling helpers.

    python -m efanna_gb300.profiling table <ncu.csv>        per-kernel launch counts, time, share
    python -m efanna_gb300.profiling search [--n N] [--nq Q] [--point E P X] [--trees T]
                                            [--precision fp32|bf16|fp8 ...] [--repeat R]
                                            [--method 0|1] [--recall] [--phase-clocks]
        builds a graph on the seeded mixture and runs batched searches (R per precision and
        point): the small case used for Nsight Compute captures of nnexp_kernel (N=400k keeps
        the base above the L2 size).  --phase-clocks runs the same searches on the diagnostic
        build of the library (EFG_PHASE_CLOCKS: every CTA of nnexp_kernel reports the SM cycles
        of each phase) and prints each search's phase shares after its line.
    python -m efanna_gb300.profiling build [--n N] [--dim D] [--data u8|unit|aniso] [--K K] [--L L]
                                           [--check C] [--S S] [--trees T] [--ml M] [--iter I]
        builds the graph of one configuration from host data (the base drawn on the GPU for the
        unit and aniso generators and copied back) and reports the build's phases and the graph
        recall@K of 2000 sampled rows against their exact neighbours.
    python -m efanna_gb300.profiling mlp [--n N] [--queries Q]
        the learned form's prediction on the tensor cores: a 96-d anisotropic index of N points,
        an untrained network (96-256-256-(1024 + 8)), Q queries predicted three times, and the
        prediction rate.
    python -m efanna_gb300.profiling knn [--n N] [--nq Q] [--dim D] [--k K] [--data u8|unit]
                                         [--screening auto|fp32|split] [--repeat R]
        times the exact k-NN (tensor-core or FP32 screening) on seeded data: per call the
        library's event times of the conversion, the screening kernel and the merge, and the
        screening's TFLOP/s against the measured BF16 peak.
"""
from __future__ import annotations

import argparse
import collections
import ctypes
import csv
import os
import subprocess
import sys

import numpy as np

_SCALE = {"ns": 1e-6, "nsecond": 1e-6, "us": 1e-3, "usecond": 1e-3, "ms": 1.0, "msecond": 1.0, "s": 1e3,
          "second": 1e3}


def launch_table(path: str, metric: str = "gpu__time_duration.sum"):
    rows = list(csv.reader(open(path)))
    start = next(i for i, r in enumerate(rows) if r and r[0] == "ID")
    hdr = rows[start]
    ki, ni, ui, vi = (hdr.index(c) for c in ("Kernel Name", "Metric Name", "Metric Unit", "Metric Value"))
    agg = collections.OrderedDict()
    for r in rows[start + 1:]:
        if len(r) <= vi or r[ni] != metric:
            continue
        name = r[ki].split("(")[0].replace("void ", "")
        ms = float(r[vi].replace(",", "")) * _SCALE[r[ui]]
        a = agg.setdefault(name, [0, 0.0])
        a[0] += 1
        a[1] += ms
    total = sum(v[1] for v in agg.values())
    out = ["| kernel | launches | total ms | share |", "|---|---|---|---|"]
    for name, (n, ms) in sorted(agg.items(), key=lambda kv: -kv[1][1]):
        out.append("| `%s` | %d | %.3f | %.2f%% |" % (name, n, ms, 100.0 * ms / total))
    out.append("| total | %d | %.3f | 100%% |" % (sum(v[0] for v in agg.values()), total))
    return "\n".join(out)


def idx_exact(x, q):
    """Exact 10-NN on the GPU (the library's brute force)."""
    import torch

    import efanna_gb300 as E
    X, Q = torch.from_numpy(x).cuda(), torch.from_numpy(q).cuda()
    out = torch.zeros((q.shape[0], 10), dtype=torch.int32, device="cuda")
    E.brute_force_knn_device(X.data_ptr(), x.shape[0], x.shape[1], x.shape[1], Q.data_ptr(), q.shape[0], q.shape[1],
                             10, out.data_ptr())
    torch.cuda.synchronize()
    return out.cpu().numpy()


def knn_case(n: int, nq: int, dim: int, k: int, data: str, screening: str, repeat: int) -> None:
    import json
    import time

    import torch

    import efanna_gb300 as E
    from efanna_gb300 import datasets
    if data == "u8":
        x = datasets.mixture_u8(n, dim, seed=0)
        q = datasets.mixture_u8(nq, dim, seed=0, queries=True)
    else:
        x = datasets.mixture_unit(n, dim, block=16, seed=0)
        q = datasets.mixture_unit(nq, dim, block=16, seed=0, queries=True)
    X, Q = torch.from_numpy(x).cuda(), torch.from_numpy(q).cuda()
    ids = torch.zeros((nq, k), dtype=torch.int32, device="cuda")
    peak = None
    pk = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "MEASURED_PEAKS.json")
    if os.path.exists(pk):
        peak = float(json.load(open(pk))["bf16_tflops"])
    for r in range(repeat):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        E.brute_force_knn_device(X.data_ptr(), n, dim, dim, Q.data_ptr(), nq, dim, k, ids.data_ptr(),
                                 screening=screening)
        torch.cuda.synchronize()
        wall = (time.perf_counter() - t0) * 1e3
        if screening == "fp32":
            print("knn fp32 %d x %d, %d queries, k=%d: wall %.2f ms" % (n, dim, nq, k, wall))
            continue
        st = E.knn_stats()
        tf = st.screen_flops / (st.screen_ms * 1e-3) / 1e12
        tt = st.tile_flops / (st.screen_ms * 1e-3) / 1e12
        print("knn %s %d x %d, %d queries, k=%d: convert %.3f ms, bound %.3f ms (%d sample rows), screen %.3f ms "
              "(%.1f TFLOP/s algorithmic, %.1f issued%s), merge %.3f ms, wall %.2f ms; terms %d, stages %d, "
              "chunks %d, CTAs %d"
              % (screening, n, dim, nq, k, st.convert_ms, st.bound_ms, st.sample_rows, st.screen_ms, tf, tt,
                 (", %.3f of measured %.0f" % (tt / peak, peak)) if peak else "", st.merge_ms, wall, st.terms,
                 st.stages, st.nchunks, st.ctas))


def make_base(n: int, dim: int, data: str, seed: int = 0, queries: bool = False):
    """Host float32 rows of one of the seeded generators."""
    from efanna_gb300 import datasets
    if data == "u8":
        return datasets.mixture_u8(n, dim, seed=seed, queries=queries)
    if data == "unit":
        return datasets.mixture_unit_device(n, dim, seed=seed, queries=queries).cpu().numpy()
    return datasets.mixture_aniso_device(n, dim, seed=seed, queries=queries).cpu().numpy()


def build_case(n: int, dim: int, data: str, K: int, L: int, check: int, S: int, trees: int, ml: int,
               iters: int, precisions=("fp32",)) -> None:
    import time

    import torch

    import efanna_gb300 as E
    t0 = time.perf_counter()
    x = make_base(n, dim, data)
    gen_s = time.perf_counter() - t0
    X = torch.from_numpy(x).cuda()
    rows = np.sort(np.random.default_rng(3).choice(n, min(n, 2000), replace=False))
    S_ = X[torch.from_numpy(rows).cuda()].contiguous()
    gt = torch.zeros((len(rows), K + 1), dtype=torch.int32, device="cuda")
    E.brute_force_knn_device(X.data_ptr(), n, dim, dim, S_.data_ptr(), len(rows), dim, K + 1, gt.data_ptr())
    torch.cuda.synchronize()
    gtn = gt.cpu().numpy()
    for prec in precisions:
        idx = E.Index(x, E.IndexParams(trees=trees, merge_level=ml, epochs=iters, check=check, L=L, K=K, S=S))
        idx.set_build_precision(prec)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        idx.build_index()
        torch.cuda.synchronize()
        build_s = time.perf_counter() - t0
        st = idx.build_stats()
        g = idx.graph()
        # the sampled rows are base rows: each one's exact K neighbours other than itself
        rec = np.mean([len(set(g[r].tolist()) & set([v for v in gtn[i] if v != r][:K])) / K
                       for i, r in enumerate(rows)])
        print("build %s %d x %d K=%d L=%d check=%d S=%d trees=%d ml=%d iter=%d join %s: data %.1f s, build %.3f s "
              "(trees %.1f ms, init %.1f ms, refine %.1f ms), join pairs %d, records %d, nodes larger than a tile %d; "
              "graph recall@%d (2000 rows) %.4f"
              % (data, n, dim, K, L, check, S, trees, ml, iters, prec, gen_s, build_s, st.trees_ms, st.init_ms,
                 st.refine_ms, st.join_pairs, st.join_records, st.join_large_nodes, K, rec), flush=True)
        idx.close()


def mlp_case(n: int, nq: int) -> None:
    import time

    import torch

    import efanna_gb300 as E
    from efanna_gb300 import datasets
    X = datasets.mixture_aniso_device(n, 96, seed=0)
    Q = datasets.mixture_aniso_device(nq, 96, seed=0, queries=True)
    idx = E.Index.from_device(X.data_ptr(), n, 96, 96, E.IndexParams(trees=4, merge_level=4, epochs=2, K=10))
    idx.build_index()
    idx.build_trees(4)
    L = E.Learned(idx, clusters=1024, entries_per_cluster=8, entry_clusters=8, hidden=256,
                  rungs=[(4, 200, 20), (4, 400, 40), (4, 600, 60), (4, 800, 80), (4, 1000, 100), (4, 1500, 150),
                         (4, 2000, 200), (4, 3000, 300)], kmeans_iters=2, kmeans_sample=20000)
    rung = torch.zeros(nq, dtype=torch.int32, device="cuda")
    cl = torch.zeros((nq, 8), dtype=torch.int32, device="cuda")
    for r in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        L.predict_device(Q.data_ptr(), nq, 96, cl.data_ptr(), rung.data_ptr(), 0, 0.9)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        print("mlp predict %d queries: %.3f ms, %.1f M queries/s" % (nq, dt * 1e3, nq / dt / 1e6), flush=True)
    L.close()
    idx.close()


def search_case(n: int, nq: int, point, trees: int, extra=None, precisions=("fp32",), repeat: int = 2,
                method: int = 0, recall: bool = False) -> None:
    import time

    import efanna_gb300 as E
    from efanna_gb300 import datasets
    x = datasets.mixture_u8(n, 128, seed=0)
    q = datasets.mixture_u8(nq, 128, seed=0, queries=True)
    idx = E.Index(x, E.IndexParams(trees=8, merge_level=8, epochs=8, check=25, L=30, K=10, S=10))
    idx.build_index()
    idx.build_trees(trees)
    pts = [point] + list(extra or [])
    gt = None
    if recall:
        gt = idx_exact(x, q)
    for prec in precisions:
        idx.set_search_precision(prec)
        for pt in pts:
            for _ in range(repeat):
                idx.set_search_params(pt[0], pt[1], pt[2], trees, -1, method)  # kgraph enlarges the pool
                t0 = time.perf_counter()
                res = idx.knn_search(10, q)
                s = idx.search_stats()
                wall = time.perf_counter() - t0
                rec = "" if gt is None else ", recall@10 %.4f" % np.mean(
                    [len(set(r) & set(g)) / 10 for r, g in zip(res, gt)])
                # the diagnostic build's device printf lines sit in the C library's stdout buffer: push them
                # out before this search's line so that each search's counters precede its line
                ctypes.CDLL(None).fflush(None)
                print("search %s method %d %d/%d/%d, %d queries: %.3f ms kernel (%d launches), %.1f evals/query, "
                      "%.1f expanded/query, %d overflow, wall %.3f s%s" %
                      (prec, method, pt[0], pt[1], pt[2], nq, s.device_ms, s.kernel_launches, s.distance_evals / nq,
                       s.expanded_nodes / nq, s.overflow_queries, wall, rec), flush=True)


PHASES = ("setup", "tree descent", "leaf-sequence scan", "pool fill", "pool distances", "pool folds",
          "expansion", "epoch distances", "epoch folds", "output", "rest")


def phase_summary(lines) -> str:
    """Sums the diagnostic build's per-CTA lines ("EFG_PHASE threads queries c0 .. c10") into
    per-phase shares and cycles per query."""
    tot = np.zeros(len(PHASES))
    queries = 0
    for ln in lines:
        f = ln.split()
        queries += int(f[2])
        tot += np.array([float(v) for v in f[3:3 + len(PHASES)]])
    if queries == 0 or tot.sum() == 0:
        return "  (no phase counters)"
    out = ["  %d CTAs, %d queries, %.0f CTA cycles per query" % (len(lines), queries, tot.sum() / queries)]
    for name, c in zip(PHASES, tot):
        out.append("  %-20s %6.1f%%  %9.1f kcycles/query" % (name, 100 * c / tot.sum(), c / queries / 1e3))
    return "\n".join(out)


def run_phase_clocks(argv) -> int:
    """Builds the diagnostic library, reruns this search command on it and summarises the phase
    counters printed before each search's line."""
    from . import build as _b
    lib = _b.build(phase_clocks=True)
    env = dict(os.environ, EFG_LIBRARY=lib)
    args = [a for a in argv if a != "--phase-clocks"]
    r = subprocess.run([sys.executable, "-m", "efanna_gb300.profiling"] + args, env=env, capture_output=True,
                       text=True)
    pending = []
    for ln in r.stdout.splitlines():
        if ln.startswith("EFG_PHASE "):
            pending.append(ln)
        else:
            print(ln)
            if ln.startswith("search "):
                print(phase_summary(pending))
                pending = []
    sys.stderr.write(r.stderr)
    return r.returncode


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    sub = ap.add_subparsers(dest="cmd")
    t = sub.add_parser("table")
    t.add_argument("csv")
    s = sub.add_parser("search")
    s.add_argument("--n", type=int, default=400000)
    s.add_argument("--nq", type=int, default=2000)
    s.add_argument("--point", type=int, nargs=3, default=[8, 6000, 600])
    s.add_argument("--trees", type=int, default=16)
    s.add_argument("--also", type=int, nargs=3, action="append", default=[],
                   help="further epochs/pool/extend points to time after --point")
    s.add_argument("--precision", nargs="+", default=["fp32"], choices=["fp32", "bf16", "fp8"])
    s.add_argument("--repeat", type=int, default=2)
    s.add_argument("--method", type=int, default=0, help="0 nnexp, 1 kgraph")
    s.add_argument("--recall", action="store_true", help="also report recall@10 against the exact 10-NN")
    s.add_argument("--phase-clocks", action="store_true",
                   help="run on the diagnostic build and print per-phase cycle shares of nnexp_kernel")
    b = sub.add_parser("build")
    b.add_argument("--n", type=int, default=1000000)
    b.add_argument("--dim", type=int, default=128)
    b.add_argument("--data", default="u8", choices=["u8", "unit", "aniso"])
    b.add_argument("--K", type=int, default=10)
    b.add_argument("--L", type=int, default=30)
    b.add_argument("--check", type=int, default=25)
    b.add_argument("--S", type=int, default=10)
    b.add_argument("--trees", type=int, default=8)
    b.add_argument("--ml", type=int, default=8)
    b.add_argument("--iter", type=int, default=8)
    b.add_argument("--precision", nargs="+", default=["fp32"], choices=["fp32", "bf16"],
                   help="join precision(s) to build with, one build each")
    ml = sub.add_parser("mlp")
    ml.add_argument("--n", type=int, default=200000)
    ml.add_argument("--queries", type=int, default=100000)
    kn = sub.add_parser("knn")
    kn.add_argument("--n", type=int, default=1000000)
    kn.add_argument("--nq", type=int, default=10000)
    kn.add_argument("--dim", type=int, default=128)
    kn.add_argument("--k", type=int, default=10)
    kn.add_argument("--data", default="u8", choices=["u8", "unit"])
    kn.add_argument("--screening", default="auto", choices=["auto", "fp32", "split"])
    kn.add_argument("--repeat", type=int, default=3)
    a = ap.parse_args()
    if a.cmd == "mlp":
        mlp_case(a.n, a.queries)
    elif a.cmd == "build":
        build_case(a.n, a.dim, a.data, a.K, a.L, a.check, a.S, a.trees, a.ml, a.iter, a.precision)
    elif a.cmd == "knn":
        knn_case(a.n, a.nq, a.dim, a.k, a.data, a.screening, a.repeat)
    elif a.cmd == "table":
        print(launch_table(a.csv))
    elif a.cmd == "search" and a.phase_clocks:
        sys.exit(run_phase_clocks(sys.argv[1:]))
    elif a.cmd == "search":
        search_case(a.n, a.nq, a.point, a.trees, a.also, a.precision, a.repeat, a.method, a.recall)
    else:
        ap.print_help()
        sys.exit(1)
