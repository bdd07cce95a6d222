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


def _declarations():
    """(return type, name, argument count) of every function the header declares."""
    txt = open(HEADER).read()
    out = []
    for ret, name, args in re.findall(r"^(int|void|uint64_t|uint32_t|const char\*)\s+(efg_[a-z0-9_]+)\s*\(([^)]*)\)",
                                      txt, re.M):
        out.append((ret, name, 0 if args.strip() in ("", "void") else args.count(",") + 1))
    return out


def test_every_entry_point_refuses_null_arguments(efg):
    """Each status-returning entry point called with every argument zero (null handles, null
    pointers, zero sizes) returns EFG_ERR_ARG with a message, before any GPU work; the getters
    return 0 and the destroy/default functions accept null.  Runs here, with no GPU."""
    import ctypes as C
    lib = C.CDLL(efg.LIB_PATH)  # no argtypes: 64-bit zeros fill pointer and integer slots alike
    lib.efg_last_error.restype = C.c_char_p
    decls = _declarations()
    assert len(decls) >= 50
    for ret, name, nargs in decls:
        f = getattr(lib, name)
        zeros = [C.c_uint64(0)] * nargs
        if name in ("efg_last_error", "efg_version"):
            continue
        if ret == "int":
            f.restype = C.c_int
            rc = f(*zeros)
            if name == "efg_search_plan_threads":  # a thread count, 0 for no plan
                assert rc == 0
                continue
            assert rc == efg.EFG_ERR_ARG, (name, rc)
            assert lib.efg_last_error(), name
        elif ret in ("uint64_t", "uint32_t"):
            f.restype = C.c_uint64 if ret == "uint64_t" else C.c_uint32
            assert f(*zeros) == 0, name
        else:
            f.restype = None
            f(*zeros)


def test_index_close_destroys_its_dependents_first(efg, monkeypatch):
    """Closing an Index first closes the plans, learned models and hash tables built on it (the
    library requires the index to outlive them); objects of another index stay open.  The C
    library is replaced by a recorder, so this runs without a GPU."""
    import ctypes as C
    calls = []

    class FakeLib:
        def __getattr__(self, name):
            return lambda h: calls.append((name, h.value if isinstance(h, C.c_void_p) else h))

    monkeypatch.setattr(efg, "lib", lambda: FakeLib())
    idx, other = object.__new__(efg.Index), object.__new__(efg.Index)
    idx._h, other._h = C.c_void_p(0x1000), C.c_void_p(0x2000)
    made = []
    for cls, h, owner in ((efg.Learned, 0x11, idx), (efg.SearchPlan, 0x12, idx), (efg.HashTables, 0x13, idx),
                          (efg.HashTables, 0x23, other)):
        o = object.__new__(cls)
        o.index, o._h = owner, C.c_void_p(h)
        efg._live[{"Learned": "learned", "SearchPlan": "plan", "HashTables": "hash"}[cls.__name__]].add(o)
        made.append(o)
    idx.close()
    assert calls == [("efg_learned_destroy", 0x11), ("efg_search_plan_destroy", 0x12),
                     ("efg_hash_destroy", 0x13), ("efg_index_destroy", 0x1000)]
    idx.close()                                   # idempotent
    assert len(calls) == 4
    other.close()
    assert calls[4:] == [("efg_hash_destroy", 0x23), ("efg_index_destroy", 0x2000)]
    for o in made:
        efg._live["learned"].discard(o), efg._live["plan"].discard(o), efg._live["hash"].discard(o)


def test_phase_clock_build_exports_the_same_symbols(efg):
    """The diagnostic build (per-phase cycle counters in the search kernel) compiles beside the
    product library, under its own name, with the same entry points."""
    import shutil
    from efanna_gb300 import build as B
    if not (os.environ.get("NVCC") or shutil.which("nvcc") or os.path.exists("/usr/local/cuda/bin/nvcc")):
        pytest.skip("nvcc not available")
    lib = B.build(phase_clocks=True)
    assert lib == B.PHASE_LIB and lib != B.LIB
    syms = []
    for path in (B.LIB, lib):
        out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True).stdout
        syms.append(set(re.findall(r" T (efg_[a-z0-9_]+)", out)))
    assert syms[0] == syms[1] and set(declared()) <= syms[1]
