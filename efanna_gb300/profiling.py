"""Summaries of Nsight Compute CSV output (per-kernel launch counts, total time and share)."""
from __future__ import annotations

import collections
import csv
import sys

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


if __name__ == "__main__":
    print(launch_table(sys.argv[1]))
