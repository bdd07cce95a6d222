"""The drop-in boundary without a GPU: the reference's own sample programs compile unchanged
against include/efanna_gb300/efanna.hpp and link against libefanna_gb300.so."""
import os
import subprocess

import pytest

from conftest import ROOT

REF = "/root/reference"
SAMPLES = ["efanna_index_buildgraph", "efanna_index_buildtrees", "efanna_index_buildall", "efanna_search"]


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "samples")), reason="reference sources not present")
@pytest.mark.parametrize("sample", SAMPLES)
def test_reference_sample_compiles_against_facade(efg, sample, tmp_path):
    src = os.path.join(REF, "samples", sample + ".cc")
    out = str(tmp_path / sample)
    cmd = ["g++", "-std=c++11", "-O1", "-w", "-I", os.path.join(ROOT, "include", "efanna_gb300"),
           "-I", os.path.join(ROOT, "oracle", "shim"), src, "-L", os.path.dirname(efg.LIB_PATH), "-lefanna_gb300",
           "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    nm = subprocess.run(["nm", "-u", out], capture_output=True, text=True).stdout
    assert "efg_index_create" in nm


def test_cli_builds_and_prints_usage(efg):
    from efanna_gb300 import build
    cli = build.build_cli()
    r = subprocess.run([cli], capture_output=True, text=True)
    assert r.returncode == 1 and "efanna_search" in r.stderr
    r = subprocess.run([cli, "evaluate"], capture_output=True, text=True)
    assert r.returncode == 255 and "gound_truth" in r.stdout


def build_hashing_driver(efg, out_dir):
    """oracle/ref_drivers/hashing_search.cc -- a program written against the reference's API
    (HASHINGIndexParams, FIndex) -- compiled against the facade instead of the reference."""
    src = os.path.join(ROOT, "oracle", "ref_drivers", "hashing_search.cc")
    out = os.path.join(str(out_dir), "hashing_search_gb300")
    cmd = ["g++", "-std=c++11", "-O1", "-w", "-I", os.path.join(ROOT, "include", "efanna_gb300"), src,
           "-L", os.path.dirname(efg.LIB_PATH), "-lefanna_gb300", "-Wl,-rpath," + os.path.dirname(efg.LIB_PATH),
           "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def test_hashing_program_compiles_against_facade(efg, tmp_path):
    out = build_hashing_driver(efg, tmp_path)
    nm = subprocess.run(["nm", "-u", out], capture_output=True, text=True).stdout
    assert "efg_hash_create" in nm and "efg_hash_search" in nm


def build_nnexp_driver(efg, out_dir):
    """oracle/ref_drivers/nnexp_search.cc -- the calls of the reference's efanna_search in a
    program of this project -- compiled against the facade instead of the reference."""
    src = os.path.join(ROOT, "oracle", "ref_drivers", "nnexp_search.cc")
    out = os.path.join(str(out_dir), "nnexp_search_gb300")
    cmd = ["g++", "-std=c++11", "-O1", "-w", "-I", os.path.join(ROOT, "include", "efanna_gb300"), src,
           "-L", os.path.dirname(efg.LIB_PATH), "-lefanna_gb300", "-Wl,-rpath," + os.path.dirname(efg.LIB_PATH),
           "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def golden_search_files(case, tmp_path):
    """The case's base and queries as fvecs, its trees and graph files and search parameters."""
    import numpy as np
    from conftest import GOLDEN, load_golden
    from efanna_gb300 import io
    g = load_golden(case)
    bf, qf = str(tmp_path / "b.fvecs"), str(tmp_path / "q.fvecs")
    io.write_fvecs(bf, g["base"].astype(np.float32))
    io.write_fvecs(qf, g["queries"].astype(np.float32))
    st, se, pool, ext, k = [str(int(v)) for v in g["search_params"]]
    args = [bf, os.path.join(GOLDEN, case + ".trees"), os.path.join(GOLDEN, case + ".graph"), qf]
    return g, args, [st, se, pool, ext, k]


def test_nnexp_driver_compiles_against_facade(efg, tmp_path):
    out = build_nnexp_driver(efg, tmp_path)
    nm = subprocess.run(["nm", "-u", out], capture_output=True, text=True).stdout
    assert "efg_knn_search" in nm and "efg_load_trees" in nm


@pytest.mark.parametrize("case", ["small_d32", "mid_d128"])
def test_nnexp_driver_on_reference_writes_golden_results(case, tmp_path):
    """The driver compiled against the reference's own headers writes the reference's results
    file (that of its efanna_search, tests/golden) byte for byte: the driver's calls are the
    sample's.  Needs the reference programs built by `make -C oracle ref` (where the sources are)."""
    import numpy as np
    from oracle import ref_bin
    from efanna_gb300 import io
    exe = ref_bin("nnexp_search", "strict")
    if exe is None:
        pytest.skip("reference drivers not built (reference sources absent)")
    g, files, params = golden_search_files(case, tmp_path)
    res = str(tmp_path / "r.ivecs")
    r = subprocess.run([exe] + files + [res] + params, capture_output=True, text=True,
                       env=dict(os.environ, OMP_NUM_THREADS="1"))
    assert r.returncode == 0, r.stdout + r.stderr
    assert np.array_equal(io.read_ivecs(res), g["results"])
    k = int(params[-1])
    ref_bytes = np.concatenate([np.full((len(g["results"]), 1), k, np.int32), g["results"]], 1).tobytes()
    assert open(res, "rb").read() == ref_bytes
