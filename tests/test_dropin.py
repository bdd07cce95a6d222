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
