"""Host logic of the profiling helpers: the ncu launch-list table behind the launch summaries and the
phase-counter summary of the diagnostic build (no GPU)."""
import os
import tempfile

import pytest

from efanna_gb300 import profiling as P


def test_launch_table_sums_launches_and_shares():
    csv_text = "\n".join([
        "==PROF== Connected to process 1",
        '"ID","Process ID","Process Name","Host Name","Kernel Name","Context","Stream","Block Size",'
        '"Grid Size","Device","CC","Section Name","Metric Name","Metric Unit","Metric Value"',
        '"0","1","python","h","void efg::s256::nnexp_kernel(const float *)","1","7","(256, 1, 1)","(304, 1, 1)",'
        '"0","10.3","Command line profiler metrics","gpu__time_duration.sum","ms","3.000"',
        '"1","1","python","h","void efg::s256::nnexp_kernel(const float *)","1","7","(256, 1, 1)","(304, 1, 1)",'
        '"0","10.3","Command line profiler metrics","gpu__time_duration.sum","us","1,000.0"',
        '"2","1","python","h","efg::join_dist_kernel(unsigned int)","1","7","(256, 1, 1)","(608, 1, 1)",'
        '"0","10.3","Command line profiler metrics","gpu__time_duration.sum","ns","1000000"',
    ])
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "launches.csv")
        open(path, "w").write(csv_text + "\n")
        table = P.launch_table(path)
    lines = table.splitlines()
    assert lines[2] == "| `efg::s256::nnexp_kernel` | 2 | 4.000 | 80.00% |"
    assert lines[3] == "| `efg::join_dist_kernel` | 1 | 1.000 | 20.00% |"
    assert lines[-1] == "| total | 3 | 5.000 | 100% |"


def test_phase_summary_sums_ctas():
    lines = ["EFG_PHASE 256 10 " + " ".join(["100"] * 6 + ["400"] + ["100"] * 4),
             "EFG_PHASE 256 30 " + " ".join(["100"] * 6 + ["400"] + ["100"] * 4)]
    out = P.phase_summary(lines).splitlines()
    assert out[0].strip() == "2 CTAs, 40 queries, 70 CTA cycles per query"
    exp = [ln for ln in out if ln.strip().startswith("expansion")][0]
    assert "28.6%" in exp                       # 800 of 2800 cycles
    assert len(out) == 1 + len(P.PHASES)
    assert "no phase counters" in P.phase_summary([])


@pytest.mark.parametrize("bad", ["EFG_PHASE 256", "EFG_PHASE 256 x 1 2"])
def test_phase_summary_rejects_malformed_lines(bad):
    with pytest.raises((ValueError, IndexError)):
        P.phase_summary([bad])
