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
