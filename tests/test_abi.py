"""The C-ABI library: it loads here (no GPU) and exports every symbol the header declares."""
import os
import re
import subprocess

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "efanna_gb300.h")


def declared():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"\b(efg_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_declared_symbols(efg):
    lib = efg.lib()
    missing = [s for s in declared() if not hasattr(lib, s)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", efg.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (efg_[a-z0-9_]+)", out))
    assert set(declared()) <= exported


def test_default_params_match_kdtreeub_defaults(efg):
    p = efg.BuildParams()
    efg.lib().efg_default_build_params(p)
    assert (p.K, p.S, p.L, p.check_k, p.epochs, p.trees, p.merge_level, p.leaf_size, p.reverse_cap) == \
        (10, 10, 30, 25, 4, 4, 4, 10, 100)


def test_version_and_error_string(efg):
    assert "sm_103a" in efg.version()
    assert isinstance(efg.lib().efg_last_error(), bytes)


def test_argument_errors_without_gpu(efg):
    import ctypes as C
    import numpy as np
    h = C.c_void_p()
    x = np.zeros((4, 8), np.float32)
    p = efg.IndexParams(S=10).to_c()
    rc = efg.lib().efg_index_create(x.ctypes.data_as(C.POINTER(C.c_float)), 4, 8, 8, C.byref(p), C.byref(h))
    assert rc == efg.EFG_ERR_ARG  # fewer than 2*S+2 points
    rc = efg.lib().efg_index_create(None, 4, 8, 8, C.byref(p), C.byref(h))
    assert rc == efg.EFG_ERR_ARG
