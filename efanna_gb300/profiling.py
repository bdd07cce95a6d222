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
"""
from __future__ import annotations

import argparse
import collections
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
                print("search %s method %d %d/%d/%d, %d queries: %.3f ms kernel (%d launches), %.1f evals/query, "
                      "%.1f expanded/query, %d overflow, wall %.3f s%s" %
                      (prec, method, pt[0], pt[1], pt[2], nq, s.device_ms, s.kernel_launches, s.distance_evals / nq,
                       s.expanded_nodes / nq, s.overflow_queries, wall, rec))


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
    a = ap.parse_args()
    if a.cmd == "table":
        print(launch_table(a.csv))
    elif a.cmd == "search" and a.phase_clocks:
        sys.exit(run_phase_clocks(sys.argv[1:]))
    elif a.cmd == "search":
        search_case(a.n, a.nq, a.point, a.trees, a.also, a.precision, a.repeat, a.method, a.recall)
    else:
        ap.print_help()
        sys.exit(1)
