"""Builds the CUDA library (libefanna_gb300.so) in-tree for sm_103a.

Each translation unit is compiled by nvcc in parallel, then linked into one shared library next
to this file.  ``python -m efanna_gb300.build`` or ``efanna_gb300.build.build()``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libefanna_gb300.so")
# diagnostic build with per-phase cycle counters in the search kernel (EFG_PHASE_CLOCKS): its own
# objects and library name, so it never replaces the library above
PHASE_OUT_DIR = os.path.join(HERE, "_build_phase")
PHASE_LIB = os.path.join(HERE, "libefanna_gb300_phase.so")
CLI_SRC = os.path.join(HERE, "cli", "efg_cli.cc")
CLI = os.path.join(HERE, "cli", "efg_cli")
SOURCES = ["index.cu", "distance.cu", "search.cu", "kgraph.cu", "plan.cu", "learned.cu", "hashing.cu", "trees.cu", "nndescent.cu", "noalloc.cu", "gram_tc.cu", "mlp_tc.cu", "join_tc.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _flags(phase_clocks: bool = False):
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
                   "-I" + os.path.join(ROOT, "include"), "-I" + CSRC, "--expt-relaxed-constexpr"] + \
        (["-DEFG_PHASE_CLOCKS=1"] if phase_clocks else [])


def _compile(src: str, phase_clocks: bool = False) -> str:
    obj = os.path.join(PHASE_OUT_DIR if phase_clocks else OUT_DIR, os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    deps = [path] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".inc"))]
    deps.append(os.path.join(ROOT, "include", "efanna_gb300.h"))
    if os.path.exists(obj) and all(os.path.getmtime(obj) >= os.path.getmtime(d) for d in deps):
        return obj
    cmd = [nvcc(), "-c", path, "-o", obj] + _flags(phase_clocks)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
    return obj


def build(verbose: bool = False, phase_clocks: bool = False) -> str:
    """Builds the library; ``phase_clocks`` builds the diagnostic one (PHASE_LIB) instead."""
    lib = PHASE_LIB if phase_clocks else LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    if phase_clocks:
        os.makedirs(PHASE_OUT_DIR, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:  # only search.cu reads the macro
        objs = list(ex.map(lambda src: _compile(src, phase_clocks and src == "search.cu"), SOURCES))
    if os.path.exists(lib) and all(os.path.getmtime(lib) >= os.path.getmtime(o) for o in objs):
        return lib
    cmd = [nvcc(), "-shared", "-o", lib] + objs + ARCH + ["-lcudart", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    if verbose:
        print("built", lib)
    return lib


def build_cli() -> str:
    """The reference-shaped command-line tools, linked against the library (host C++ only)."""
    lib = build()
    if os.path.exists(CLI) and os.path.getmtime(CLI) >= max(os.path.getmtime(CLI_SRC), os.path.getmtime(lib)):
        return CLI
    cmd = [os.environ.get("CXX", "g++"), "-std=c++11", "-O2", CLI_SRC, "-o", CLI,
           "-I" + os.path.join(ROOT, "include", "efanna_gb300"), "-L" + HERE, "-lefanna_gb300",
           "-Wl,-rpath,$ORIGIN/.."]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("CLI build failed:\n%s%s" % (r.stdout, r.stderr))
    return CLI


if __name__ == "__main__":
    build(verbose=True)
    build_cli()
    sys.exit(0)
