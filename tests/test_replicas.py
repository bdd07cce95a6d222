"""Replica orchestration across ranks (efanna_gb300/replicas.py) with world size 2 on the CPU:
`gloo` process group, the slowest rank's time, whole-job throughput and query shares."""
import os
import socket
import subprocess
import sys
import textwrap

from efanna_gb300 import replicas

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_query_slices_partition_the_batch():
    for nq in (0, 1, 7, 10, 1001):
        for ws in (1, 2, 3, 8):
            parts = [replicas.query_slice(nq, r, ws) for r in range(ws)]
            assert parts[0][0] == 0 and parts[-1][1] == nq
            assert all(a[1] == b[0] for a, b in zip(parts, parts[1:]))
            sizes = [b - a for a, b in parts]
            assert max(sizes) - min(sizes) <= 1


def test_two_gloo_ranks_agree_on_the_slowest_time():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    code = textwrap.dedent("""
        import sys
        sys.path.insert(0, %r)
        from efanna_gb300 import replicas
        ws, rank, _ = replicas.world()
        assert replicas.init("gloo")
        replicas.barrier()
        ms = replicas.max_over_ranks(10.0 + 5.0 * rank)
        qps = replicas.throughput(1000, ms / 1e3, ws)
        print("rank", rank, ms, qps, replicas.query_slice(1001, rank, ws))
        replicas.finish()
    """ % ROOT)
    procs = []
    for r in range(2):
        env = dict(os.environ, WORLD_SIZE="2", RANK=str(r), LOCAL_RANK=str(r), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", code], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = [p.communicate(timeout=120) for p in procs]
    for p, (out, err) in zip(procs, outs):
        assert p.returncode == 0, err
    lines = sorted(o[0].strip() for o in outs)
    assert lines[0] == "rank 0 15.0 133333.33333333334 (0, 501)"
    assert lines[1] == "rank 1 15.0 133333.33333333334 (501, 1001)"
