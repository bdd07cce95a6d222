"""Host logic of bench.py that needs no GPU: the clock sampler that records SM clocks and throttle
reasons during a timed region (fed here by a stand-in nvidia-smi) and the roofline peak lookup."""
import json
import os
import time


def test_clock_sampler_reads_clocks_and_reasons(tmp_path, monkeypatch):
    smi = tmp_path / "nvidia-smi"
    smi.write_text("#!/bin/sh\n"
                   "echo '1965, 2070, Not Active, Not Active, Not Active, Active'\n"
                   "echo '1980, 2070, Not Active, Not Active, Not Active, Not Active'\n"
                   "echo '[N/A], 2070, Not Active, Active, Not Active, Not Active'\n"
                   "echo 'malformed line'\n"
                   "exec sleep 30\n")
    smi.chmod(0o755)
    monkeypatch.setenv("PATH", str(tmp_path) + os.pathsep + os.environ.get("PATH", ""))
    import bench
    cs = bench.ClockSampler()
    cs.start()
    t0 = time.time()
    while len(cs.samples) < 3 and time.time() - t0 < 10:
        time.sleep(0.05)
    r = cs.stop()
    assert r["samples"] == 3                          # the malformed line is dropped
    assert r["sm_mhz"] == 1972.5                      # median of the numeric samples
    assert r["sm_max_mhz"] == 2070.0
    assert r["reasons"] == ["hw_thermal_slowdown", "sw_power_cap"]


def test_clock_sampler_without_nvidia_smi(tmp_path, monkeypatch):
    monkeypatch.setenv("PATH", str(tmp_path))          # no nvidia-smi anywhere on PATH
    import bench
    cs = bench.ClockSampler()
    cs.start()
    r = cs.stop()
    assert r == {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}


def test_peaks_prefers_the_measured_file(tmp_path, monkeypatch):
    import bench
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    assert bench.peaks() == (6800.0, "fallback")
    (tmp_path / "MEASURED_PEAKS.json").write_text(json.dumps({"hbm_gbs": 6791.7, "bf16_tflops": 1900}))
    assert bench.peaks() == (6791.7, "measured")


def _bench(*args):
    import subprocess
    import sys
    from conftest import ROOT
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py")] + list(args), capture_output=True,
                          text=True, timeout=600, cwd=ROOT)


def test_reference_arm_line():
    """`bench.py --impl reference` (the OpenMP restatement of the reference on the host cores) at a
    small size: one JSON line with the arm's keys, the workload named by the sizes run."""
    r = _bench("--impl", "reference", "--n", "100000", "--nq", "200", "--steps", "3", "--warmup", "3",
               "--cpu-queries", "50")
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "queries/s" and line["value"] > 0
    assert line["steps"] == 3 and line["warmup"] == 3 and line["higher_is_better"] is True
    assert line["config"]["workload"].startswith("100k x 128 FP32") and "200 queries" in line["config"]["workload"]
    assert line["build"]["status"] == 0
    assert 0.9 < line["build"]["graph_recall@10"] <= 1.0 and line["build"]["graph_recall_rows"] == 2000
    assert 0.8 < line["recall@10"] <= 1.0 and line["recall_queries"] == 50
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": "queries/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}


def test_reference_arm_fails_when_the_build_fails():
    """Merge level 8 is deeper than the trees of a 1000-point base (leaves of 10 points): the build's
    status ends the arm with an error instead of timing a search on no graph.  (At 20k points the
    multi-threaded tree build's depth varies from run to run and level 8 sometimes fits.)"""
    r = _bench("--impl", "reference", "--n", "1000", "--nq", "100", "--steps", "3", "--warmup", "3")
    assert r.returncode != 0
    assert "graph build failed with status 3" in r.stderr


def test_recall_with_ties_counts_equally_near_points():
    """An id as near as the exact k-th neighbour counts as a hit; -1 and farther ids do not."""
    import numpy as np
    import bench
    base = np.array([[0.], [1.], [-1.], [2.], [5.]], np.float32)  # 1 and 2 are tied for the query 0
    q = np.array([[0.]], np.float32)
    gt = np.array([[0, 1]])
    assert bench.recall_ties(np.array([[0, 2]]), gt, base, q, k=2) == 1.0    # the tie counts
    assert bench.recall(np.array([[0, 2]]), gt, k=2) == 0.5                 # the strict recall does not
    assert bench.recall_ties(np.array([[0, 3]]), gt, base, q, k=2) == 0.5    # farther: a miss
    assert bench.recall_ties(np.array([[0, -1]]), gt, base, q, k=2) == 0.5   # not found: a miss
    rng = np.random.default_rng(0)
    x = rng.integers(0, 4, (300, 3)).astype(np.float32)
    qq = rng.integers(0, 4, (40, 3)).astype(np.float32)
    d = ((qq[:, None, :].astype(np.float64) - x[None]) ** 2).sum(-1)
    exact = np.argsort(d, axis=1, kind="stable")[:, :10]
    assert bench.recall_ties(exact, exact, x, qq) == 1.0
    shuffled = np.argsort(d + rng.random(d.shape) * 1e-3, axis=1)[:, :10]  # other members of the ties
    assert bench.recall_ties(shuffled, exact, x, qq) == 1.0
