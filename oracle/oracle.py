"""TEST INFRASTRUCTURE ONLY: ctypes access to the CPU oracle (oracle/efanna_oracle.cpp).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import this module.
``build()`` compiles the oracle with the committed Makefile; ``ref_bin()`` locates the reference's
own sample programs when they were compiled here from the reference sources.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
SEQ, CANON, OMP = 0, 1, 2


class Params(C.Structure):
    _fields_ = [(n, C.c_uint32) for n in
                ("K", "S", "L", "check_k", "epochs", "trees", "trees_build", "merge_level", "tns",
                 "reverse_cap")] + [("seed", C.c_uint64)]


def make_params(K=10, S=10, L=30, check_k=25, epochs=8, trees=8, trees_build=0, merge_level=8, tns=10,
                reverse_cap=100, seed=1998) -> Params:
    return Params(K, S, L, check_k, epochs, trees, trees_build or trees, merge_level, tns, reverse_cap, seed)


def build() -> str:
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)
    return LIB_PATH


def build_ref(ref_root: str = "/root/reference") -> bool:
    if not os.path.isdir(ref_root):
        return False
    r = subprocess.run(["make", "-s", "-C", HERE, "ref", "REF=" + ref_root, "-j8"])
    return r.returncode == 0


def ref_bin(name: str, flavour: str = "stock") -> str | None:
    p = os.path.join(HERE, "_ref", flavour, name)
    return p if os.path.isfile(p) and os.access(p, os.X_OK) else None


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        f32p, u32p, u8p, u64p, i32p = (C.POINTER(C.c_float), C.POINTER(C.c_uint32), C.POINTER(C.c_uint8),
                                       C.POINTER(C.c_uint64), C.POINTER(C.c_int32))
        L.orc_l2_avx.restype = C.c_float
        L.orc_l2_avx.argtypes = [f32p, f32p, C.c_uint64]
        L.orc_l2_scalar.restype = C.c_float
        L.orc_l2_scalar.argtypes = [f32p, f32p, C.c_uint64]
        L.orc_l2_pairs.argtypes = [f32p, C.c_uint64, C.c_uint64, u32p, u32p, C.c_uint64, C.c_int, f32p]
        L.orc_forest_build.restype = C.c_void_p
        L.orc_forest_build.argtypes = [f32p, C.c_uint64, C.c_uint32, C.c_uint64, C.c_uint32, C.c_uint32,
                                       C.c_uint32, C.c_int, C.c_uint64]
        L.orc_forest_save.argtypes = [C.c_void_p, C.c_char_p, C.c_uint32]
        L.orc_forest_load.restype = C.c_void_p
        L.orc_forest_load.argtypes = [C.c_char_p]
        L.orc_forest_trees.restype = C.c_uint32
        L.orc_forest_trees.argtypes = [C.c_void_p]
        L.orc_forest_free.argtypes = [C.c_void_p]
        L.orc_build_graph.argtypes = [f32p, C.c_uint64, C.c_uint32, C.c_uint64, C.POINTER(Params), C.c_int, u32p,
                                      C.POINTER(C.c_void_p), u64p]
        state = [f32p, u32p, u8p, u32p, u32p, f32p, f32p, u8p, u32p, u32p, u32p, u32p, C.c_uint32]
        L.orc_nnd_init.argtypes = [f32p, C.c_uint64, C.c_uint32, C.c_uint64, C.c_void_p, C.POINTER(Params),
                                   C.c_int] + state
        L.orc_nnd_iterate.argtypes = [f32p, C.c_uint64, C.c_uint32, C.c_uint64, C.POINTER(Params), C.c_int,
                                      C.c_uint32] + state + [u64p]
        L.orc_search.argtypes = [f32p, C.c_uint64, C.c_uint32, C.c_uint64, C.c_void_p, u64p, u32p, f32p,
                                 C.c_uint64, C.c_uint64, C.c_int, C.c_int, C.c_int, C.c_int, C.c_uint32, C.c_int,
                                 C.c_int, C.c_uint64, i32p, u64p]
        L.orc_search_batch.argtypes = [f32p, C.c_uint64, C.c_uint32, C.c_uint64, C.c_void_p, u64p, u32p, f32p,
                                       C.c_uint64, C.c_uint64, i32p, C.c_uint32, C.c_int, u32p, C.c_uint32, C.c_int,
                                       C.c_uint64, i32p]
        L.orc_search_kgraph.argtypes = [f32p, C.c_uint64, C.c_uint32, C.c_uint64, C.c_void_p, u64p, u32p, f32p,
                                        C.c_uint64, C.c_uint64, C.c_int, C.POINTER(C.c_int), C.c_int, C.c_int,
                                        C.c_uint32, C.c_int, C.c_int, C.c_uint64, i32p, u64p]
        L.orc_search_hashed.argtypes = [f32p, C.c_uint64, C.c_uint32, C.c_uint64, u64p, u32p, f32p, C.c_uint64,
                                        C.c_uint64, u64p, u64p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_int, C.c_int,
                                        C.c_int, C.c_uint32, C.c_int, C.c_int, C.c_uint64, i32p, u64p]
        L.orc_search_hashed_kgraph.argtypes = [f32p, C.c_uint64, C.c_uint32, C.c_uint64, u64p, u32p, f32p,
                                               C.c_uint64, C.c_uint64, u64p, u64p, C.c_uint32, C.c_uint32,
                                               C.c_uint32, C.c_int, C.POINTER(C.c_int), C.c_int, C.c_uint32, C.c_int,
                                               C.c_int, C.c_uint64, i32p, u64p]
        L.orc_search_hashed_buckets.argtypes = [f32p, C.c_uint64, C.c_uint32, C.c_uint64, f32p, C.c_uint64,
                                                C.c_uint64, u64p, u64p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_int,
                                                C.c_uint32, C.c_int, C.c_int, C.c_uint64, i32p]
        _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


def l2(a: np.ndarray, b: np.ndarray, order: str = "avx") -> float:
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    f = lib().orc_l2_avx if order == "avx" else lib().orc_l2_scalar
    return float(f(_p(a, C.c_float), _p(b, C.c_float), a.size))


def l2_pairs(base: np.ndarray, ia: np.ndarray, ib: np.ndarray, order: str = "avx") -> np.ndarray:
    base = np.ascontiguousarray(base, np.float32)
    ia = np.ascontiguousarray(ia, np.uint32)
    ib = np.ascontiguousarray(ib, np.uint32)
    out = np.empty(ia.size, np.float32)
    lib().orc_l2_pairs(_p(base, C.c_float), base.shape[1], base.shape[1], _p(ia, C.c_uint32), _p(ib, C.c_uint32),
                       ia.size, 0 if order == "avx" else 1, _p(out, C.c_float))
    return out


class Forest:
    def __init__(self, handle):
        self.h = handle

    @classmethod
    def build(cls, data: np.ndarray, trees: int, S: int = 10, tns: int = 10, mode: int = CANON, seed: int = 1998):
        data = np.ascontiguousarray(data, np.float32)
        h = lib().orc_forest_build(_p(data, C.c_float), data.shape[0], data.shape[1], data.shape[1], trees, S, tns,
                                   mode, seed)
        return cls(h)

    @classmethod
    def load(cls, path: str):
        h = lib().orc_forest_load(path.encode())
        if not h:
            raise IOError("cannot load trees file " + path)
        return cls(h)

    def save(self, path: str, K: int = 10) -> None:
        if lib().orc_forest_save(self.h, path.encode(), K) != 0:
            raise IOError(path)

    @property
    def trees(self) -> int:
        return int(lib().orc_forest_trees(self.h))

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_forest_free(self.h)
            self.h = None


def build_graph(data: np.ndarray, params: Params, mode: int = CANON):
    """-> (status, gs[n, K] uint32, Forest, pairs)."""
    data = np.ascontiguousarray(data, np.float32)
    n = data.shape[0]
    gs = np.zeros((n, params.K), np.uint32)
    fh = C.c_void_p()
    stats = np.zeros(2, np.uint64)
    rc = lib().orc_build_graph(_p(data, C.c_float), n, data.shape[1], data.shape[1], C.byref(params), mode,
                               _p(gs, C.c_uint32), C.byref(fh), _p(stats, C.c_uint64))
    return rc, gs, Forest(fh.value), int(stats[0] if rc == 0 else stats[1])


class NNDState:
    """Explicit NN-descent state arrays shared by the oracle and the CUDA state-level tests."""

    def __init__(self, n: int, L: int, cap: int):
        P = L + 1
        self.n, self.Lcap, self.cap = n, L, cap
        self.pool_dist = np.zeros((n, P), np.float32)
        self.pool_id = np.zeros((n, P), np.uint32)
        self.pool_flag = np.zeros((n, P), np.uint8)
        self.L = np.zeros(n, np.uint32)
        self.Range = np.zeros(n, np.uint32)
        self.radius = np.zeros(n, np.float32)
        self.radiusM = np.zeros(n, np.float32)
        self.found = np.zeros(n, np.uint8)
        self.new_ids = np.zeros((n, cap), np.uint32)
        self.new_cnt = np.zeros(n, np.uint32)
        self.old_ids = np.zeros((n, cap), np.uint32)
        self.old_cnt = np.zeros(n, np.uint32)

    FIELDS = ("pool_dist", "pool_id", "pool_flag", "L", "Range", "radius", "radiusM", "found", "new_ids",
              "new_cnt", "old_ids", "old_cnt")

    def copy(self):
        s = NNDState.__new__(NNDState)
        s.n, s.Lcap, s.cap = self.n, self.Lcap, self.cap
        for f in self.FIELDS:
            setattr(s, f, getattr(self, f).copy())
        return s

    def args(self):
        t = {np.float32: C.c_float, np.uint32: C.c_uint32, np.uint8: C.c_uint8}
        return [_p(getattr(self, f), t[getattr(self, f).dtype.type]) for f in self.FIELDS] + [self.cap]


def nnd_init(data: np.ndarray, forest: Forest, params: Params, cap: int, mode: int = CANON):
    data = np.ascontiguousarray(data, np.float32)
    st = NNDState(data.shape[0], params.L, cap)
    rc = lib().orc_nnd_init(_p(data, C.c_float), data.shape[0], data.shape[1], data.shape[1], forest.h,
                            C.byref(params), mode, *st.args())
    return rc, st


def nnd_iterate(data: np.ndarray, st: NNDState, params: Params, it: int, mode: int = CANON):
    data = np.ascontiguousarray(data, np.float32)
    out = st.copy()
    pairs = np.zeros(1, np.uint64)
    rc = lib().orc_nnd_iterate(_p(data, C.c_float), data.shape[0], data.shape[1], data.shape[1], C.byref(params),
                               mode, it, *out.args(), _p(pairs, C.c_uint64))
    if rc != 0:
        raise RuntimeError("orc_nnd_iterate failed: %d" % rc)
    return out, int(pairs[0])


def graph_csr_from_dense(gs: np.ndarray):
    n, k = gs.shape
    return (np.arange(n + 1, dtype=np.uint64) * k), np.ascontiguousarray(gs.reshape(-1), np.uint32)


def search(data, forest: Forest, gptr, gids, queries, k=10, epochs=4, init_num=1200, extend_to=200, trees=16,
           mode: int = CANON, threads: int = 1, seed: int = 1998, want_evals=False):
    data = np.ascontiguousarray(data, np.float32)
    queries = np.ascontiguousarray(queries, np.float32)
    gptr = np.ascontiguousarray(gptr, np.uint64)
    gids = np.ascontiguousarray(gids, np.uint32)
    nq = queries.shape[0]
    out = np.zeros((nq, k), np.int32)
    ev = np.zeros(nq, np.uint64)
    rc = lib().orc_search(_p(data, C.c_float), data.shape[0], data.shape[1], data.shape[1], forest.h,
                          _p(gptr, C.c_uint64), _p(gids, C.c_uint32), _p(queries, C.c_float), nq, queries.shape[1],
                          epochs, init_num, extend_to, trees, k, mode, threads, seed, _p(out, C.c_int32),
                          _p(ev, C.c_uint64))
    if rc != 0:
        raise ValueError("orc_search rejected its arguments")
    return (out, ev) if want_evals else out


def search_batch(data, forest: Forest, gptr, gids, queries, params, k_max, trees=16, seeds=None, threads=1,
                 seed: int = 1998):
    """Canonical nnexp with per-query (epochs, pool, extend, k) rows and optional entry seeds;
    trees=0 (forest may be None, seeds required) builds pools from the seeds and the random fill."""
    data = np.ascontiguousarray(data, np.float32)
    queries = np.ascontiguousarray(queries, np.float32)
    gptr = np.ascontiguousarray(gptr, np.uint64)
    gids = np.ascontiguousarray(gids, np.uint32)
    params = np.ascontiguousarray(params, np.int32).reshape(-1, 4)
    nq = queries.shape[0]
    out = np.zeros((nq, k_max), np.int32)
    sp = None if seeds is None else np.ascontiguousarray(seeds, np.uint32).reshape(nq, -1)
    rc = lib().orc_search_batch(_p(data, C.c_float), data.shape[0], data.shape[1], data.shape[1],
                                None if forest is None else forest.h,
                                _p(gptr, C.c_uint64), _p(gids, C.c_uint32), _p(queries, C.c_float), nq,
                                queries.shape[1], _p(params, C.c_int32), k_max, trees,
                                None if sp is None else _p(sp, C.c_uint32), 0 if sp is None else sp.shape[1],
                                threads, seed, _p(out, C.c_int32))
    if rc != 0:
        raise ValueError("orc_search_batch rejected its arguments")
    return out


def search_kgraph(data, forest: Forest, gptr, gids, queries, k=10, epochs=4, init_num=1200, extend_to=200,
                  trees=16, mode: int = CANON, threads: int = 1, seed: int = 1998):
    """getNeighbors_kgraph.  Returns (ids, evals per query, pool size in effect afterwards): the
    reference raises its stored pool size to epochs * extend_to when that is not smaller."""
    data = np.ascontiguousarray(data, np.float32)
    queries = np.ascontiguousarray(queries, np.float32)
    gptr = np.ascontiguousarray(gptr, np.uint64)
    gids = np.ascontiguousarray(gids, np.uint32)
    nq = queries.shape[0]
    out = np.zeros((nq, k), np.int32)
    ev = np.zeros(nq, np.uint64)
    pool = C.c_int(init_num)
    rc = lib().orc_search_kgraph(_p(data, C.c_float), data.shape[0], data.shape[1], data.shape[1], forest.h,
                                 _p(gptr, C.c_uint64), _p(gids, C.c_uint32), _p(queries, C.c_float), nq,
                                 queries.shape[1], epochs, C.byref(pool), extend_to, trees, k, mode, threads, seed,
                                 _p(out, C.c_int32), _p(ev, C.c_uint64))
    if rc != 0:
        raise ValueError("orc_search_kgraph rejected its arguments")
    return out, ev, pool.value


def search_hashed(data, gptr, gids, queries, bcodes, qcodes, bits, radius, k=10, epochs=4, init_num=1200,
                  extend_to=200, mode: int = CANON, threads: int = 1, seed: int = 1998):
    """getNeighborsIEH32_nnexp / getNeighborsIEH64_nnexp (the hashing-seeded search).  bcodes:
    tables x n, qcodes: tables x nq.  Returns (ids, evals per query)."""
    data = np.ascontiguousarray(data, np.float32)
    queries = np.ascontiguousarray(queries, np.float32)
    gptr = np.ascontiguousarray(gptr, np.uint64)
    gids = np.ascontiguousarray(gids, np.uint32)
    bcodes = np.ascontiguousarray(bcodes, np.uint64)
    qcodes = np.ascontiguousarray(qcodes, np.uint64)
    nq = queries.shape[0]
    assert bcodes.shape == (qcodes.shape[0], data.shape[0]) and qcodes.shape[1] == nq
    out = np.zeros((nq, k), np.int32)
    ev = np.zeros(nq, np.uint64)
    rc = lib().orc_search_hashed(_p(data, C.c_float), data.shape[0], data.shape[1], data.shape[1],
                                 _p(gptr, C.c_uint64), _p(gids, C.c_uint32), _p(queries, C.c_float), nq,
                                 queries.shape[1], _p(bcodes, C.c_uint64), _p(qcodes, C.c_uint64), bcodes.shape[0],
                                 bits, radius, epochs, init_num, extend_to, k, mode, threads, seed,
                                 _p(out, C.c_int32), _p(ev, C.c_uint64))
    if rc != 0:
        raise ValueError("orc_search_hashed rejected its arguments")
    return out, ev


def search_hashed_kgraph(data, gptr, gids, queries, bcodes, qcodes, bits, radius, k=10, epochs=4, init_num=1200,
                         extend_to=200, mode: int = CANON, threads: int = 1, seed: int = 1998):
    """getNeighborsIEH32_kgraph / getNeighborsIEH64_kgraph.  Returns (ids, evals per query, pool
    size in effect afterwards)."""
    data = np.ascontiguousarray(data, np.float32)
    queries = np.ascontiguousarray(queries, np.float32)
    gptr = np.ascontiguousarray(gptr, np.uint64)
    gids = np.ascontiguousarray(gids, np.uint32)
    bcodes = np.ascontiguousarray(bcodes, np.uint64)
    qcodes = np.ascontiguousarray(qcodes, np.uint64)
    nq = queries.shape[0]
    assert bcodes.shape == (qcodes.shape[0], data.shape[0]) and qcodes.shape[1] == nq
    out = np.zeros((nq, k), np.int32)
    ev = np.zeros(nq, np.uint64)
    pool = C.c_int(init_num)
    rc = lib().orc_search_hashed_kgraph(_p(data, C.c_float), data.shape[0], data.shape[1], data.shape[1],
                                        _p(gptr, C.c_uint64), _p(gids, C.c_uint32), _p(queries, C.c_float), nq,
                                        queries.shape[1], _p(bcodes, C.c_uint64), _p(qcodes, C.c_uint64),
                                        bcodes.shape[0], bits, radius, epochs, C.byref(pool), extend_to, k, mode,
                                        threads, seed, _p(out, C.c_int32), _p(ev, C.c_uint64))
    if rc != 0:
        raise ValueError("orc_search_hashed_kgraph rejected its arguments")
    return out, ev, pool.value


def search_hashed_buckets(data, queries, bcodes, qcodes, bits, radius, k=10, init_num=1200, mode: int = CANON,
                          threads: int = 1, seed: int = 1998):
    """getNeighbors32 / getNeighbors64: the hashing index's search without a graph."""
    data = np.ascontiguousarray(data, np.float32)
    queries = np.ascontiguousarray(queries, np.float32)
    bcodes = np.ascontiguousarray(bcodes, np.uint64)
    qcodes = np.ascontiguousarray(qcodes, np.uint64)
    nq = queries.shape[0]
    out = np.zeros((nq, k), np.int32)
    rc = lib().orc_search_hashed_buckets(_p(data, C.c_float), data.shape[0], data.shape[1], data.shape[1],
                                         _p(queries, C.c_float), nq, queries.shape[1], _p(bcodes, C.c_uint64),
                                         _p(qcodes, C.c_uint64), bcodes.shape[0], bits, radius, init_num, k, mode,
                                         threads, seed, _p(out, C.c_int32))
    if rc != 0:
        raise ValueError("orc_search_hashed_buckets rejected its arguments")
    return out
