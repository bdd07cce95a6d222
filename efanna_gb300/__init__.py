"""efanna_gb300 — GB300 (sm_103a) kNN-graph build and graph search behind EFANNA's index API.

Python mirror of the reference's ``FIndex<float>`` (efanna.hpp:9-75) over the C ABI declared in
include/efanna_gb300.h.  The compute runs in libefanna_gb300.so (hand-written CUDA kernels);
there is no CPU path: importing works without a GPU, but every compute call needs the library
and a CUDA device and raises ``EfannaError`` otherwise.

    idx = Index(data, IndexParams(trees=8, merge_level=8, epochs=8, check=25, L=30, K=10, S=10))
    idx.build_index()                      # buildIndex(): trees + leaf merge + NN-descent
    idx.set_search_params(epochs=4, init_num=1200, extend_to=200, search_trees=8)
    ids = idx.knn_search(10, queries)      # knnSearch()
"""
from __future__ import annotations

import atexit
import ctypes as C
import os
import weakref
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# EFG_LIBRARY selects another build of the library (the diagnostic phase-clock build)
LIB_PATH = os.environ.get("EFG_LIBRARY") or os.path.join(HERE, "libefanna_gb300.so")

EFG_OK, EFG_ERR_ARG, EFG_ERR_CUDA, EFG_ERR_MERGE_LEVEL, EFG_ERR_OPEN, EFG_ERR_FORMAT = 0, 1, 2, 3, 4, 5
EFG_ERR_STATE, EFG_ERR_TREE_COUNT, EFG_ERR_NOMEM, EFG_ERR_DEVICE_LIMIT = 6, 7, 8, 9


class EfannaError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__("efanna_gb300 error %d: %s" % (code, msg))
        self.code = code


class BuildParams(C.Structure):
    _fields_ = [(n, C.c_uint32) for n in ("K", "S", "L", "check_k", "epochs", "trees", "trees_build",
                                          "merge_level", "leaf_size", "reverse_cap")] + [("seed", C.c_uint64)]


class BuildStats(C.Structure):
    _fields_ = [("trees_ms", C.c_double), ("init_ms", C.c_double), ("refine_ms", C.c_double),
                ("total_ms", C.c_double), ("join_pairs", C.c_uint64), ("join_records", C.c_uint64),
                ("merge_distances", C.c_uint64), ("max_merge_depth", C.c_int32),
                ("join_large_nodes", C.c_uint64)]


class SearchStats(C.Structure):
    _fields_ = [("device_ms", C.c_double), ("distance_evals", C.c_uint64), ("queries", C.c_uint64),
                ("expanded_nodes", C.c_uint64), ("overflow_queries", C.c_uint64),
                ("kernel_launches", C.c_uint64), ("reranked", C.c_uint64), ("migrated_queries", C.c_uint64)]


class QueryParams(C.Structure):
    _fields_ = [("epochs", C.c_int32), ("init_num", C.c_int32), ("extend_to", C.c_int32), ("k", C.c_uint32)]


MAX_RUNGS = 16


class LearnedParams(C.Structure):
    _fields_ = [("clusters", C.c_uint32), ("kmeans_iters", C.c_uint32), ("kmeans_sample", C.c_uint32),
                ("entries_per_cluster", C.c_uint32), ("entry_clusters", C.c_uint32), ("hidden", C.c_uint32),
                ("rungs", C.c_uint32), ("rung", QueryParams * MAX_RUNGS), ("target", C.c_float),
                ("train_epochs", C.c_uint32), ("batch", C.c_uint32), ("lr", C.c_float), ("seed", C.c_uint64),
                ("trace_reference", QueryParams)]


class LearnedStats(C.Structure):
    _fields_ = [("train_queries", C.c_uint64), ("train_loss_first", C.c_float), ("train_loss_last", C.c_float),
                ("rung_recall", C.c_float * MAX_RUNGS)]


def query_params(rows) -> np.ndarray:
    """(epochs, pool, extend, k) rows -> a contiguous array laid out as efg_query_params."""
    a = np.ascontiguousarray(np.asarray(rows, dtype=np.int64).reshape(-1, 4).astype(np.int32))
    return a


class HostState(C.Structure):
    _fields_ = [("n", C.c_uint64), ("L", C.c_uint32), ("cap", C.c_uint32),
                ("pool_dist", C.POINTER(C.c_float)), ("pool_id", C.POINTER(C.c_uint32)),
                ("pool_flag", C.POINTER(C.c_uint8)), ("Lcur", C.POINTER(C.c_uint32)),
                ("Range", C.POINTER(C.c_uint32)), ("radius", C.POINTER(C.c_float)),
                ("radiusM", C.POINTER(C.c_float)), ("found", C.POINTER(C.c_uint8)),
                ("new_ids", C.POINTER(C.c_uint32)), ("new_cnt", C.POINTER(C.c_uint32)),
                ("old_ids", C.POINTER(C.c_uint32)), ("old_cnt", C.POINTER(C.c_uint32))]


@dataclass
class IndexParams:
    """KDTreeUbIndexParams(rnn_used, trees, merge_level, epoches, check, L, K, trees_build, S)
    (kdtreeub_index.hpp:14-35), with IndexParams' TNS and the update's reverse-list cap."""
    trees: int = 4
    merge_level: int = 4
    epochs: int = 4
    check: int = 25
    L: int = 30
    K: int = 10
    trees_build: int = 0
    S: int = 10
    leaf_size: int = 10
    reverse_cap: int = 100
    seed: int = 1998

    def to_c(self) -> BuildParams:
        return BuildParams(self.K, self.S, self.L, self.check, self.epochs, self.trees,
                           self.trees_build or self.trees, self.merge_level, self.leaf_size, self.reverse_cap,
                           self.seed)


_lib = None

# library objects still open, by kind: closed at interpreter exit, dependents before their index,
# while the CUDA runtime is still up (their destructors synchronise the index's stream)
_live = {"learned": weakref.WeakSet(), "plan": weakref.WeakSet(), "hash": weakref.WeakSet(),
         "index": weakref.WeakSet()}


def _close_all():
    for kind in ("learned", "plan", "hash", "index"):
        for o in list(_live[kind]):
            try:
                o.close()
            except Exception:
                pass


atexit.register(_close_all)


def lib():
    """Loads libefanna_gb300.so (building it first if it is missing and nvcc is available)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH) and LIB_PATH == os.path.join(HERE, "libefanna_gb300.so"):
        from . import build as _b
        _b.build()
    L = C.CDLL(LIB_PATH)
    vp, u64, u32, i32, f32p = C.c_void_p, C.c_uint64, C.c_uint32, C.c_int, C.POINTER(C.c_float)
    sig = {
        "efg_default_build_params": (None, [C.POINTER(BuildParams)]),
        "efg_index_create": (i32, [f32p, u64, u32, u64, C.POINTER(BuildParams), C.POINTER(vp)]),
        "efg_index_create_device": (i32, [vp, u64, u32, u64, C.POINTER(BuildParams), C.POINTER(vp)]),
        "efg_index_destroy": (None, [vp]),
        "efg_build_trees": (i32, [vp]),
        "efg_build_trees_count": (i32, [vp, u32]),
        "efg_build_graph": (i32, [vp]),
        "efg_get_build_stats": (i32, [vp, C.POINTER(BuildStats)]),
        "efg_set_search_params": (i32, [vp, i32, i32, i32, i32, i32, i32]),
        "efg_set_search_precision": (i32, [vp, i32]),
        "efg_set_build_precision": (i32, [vp, i32]),
        "efg_set_search_candidate_cap": (i32, [vp, u32]),
        "efg_screen_distances": (i32, [vp, i32, vp, u64, u64, vp, u32, vp, vp]),
        "efg_knn_search": (i32, [vp, f32p, u64, u32, u64, u32, C.POINTER(C.c_int32)]),
        "efg_knn_search_device": (i32, [vp, vp, u64, u64, u32, vp, vp]),
        "efg_get_search_stats": (i32, [vp, C.POINTER(SearchStats)]),
        "efg_save_graph": (i32, [vp, C.c_char_p]), "efg_load_graph": (i32, [vp, C.c_char_p]),
        "efg_save_trees": (i32, [vp, C.c_char_p]), "efg_load_trees": (i32, [vp, C.c_char_p]),
        "efg_save_index": (i32, [vp, C.c_char_p]), "efg_load_index": (i32, [vp, C.c_char_p]),
        "efg_save_results": (i32, [vp, C.c_char_p]),
        "efg_graph_size": (u64, [vp]),
        "efg_graph_row": (C.c_int64, [vp, u64, C.POINTER(C.c_uint32), u64]),
        "efg_graph_csr": (i32, [vp, C.POINTER(C.c_uint64), C.POINTER(C.c_uint32), C.POINTER(C.c_uint64)]),
        "efg_graph_csc": (i32, [vp, C.POINTER(C.c_uint64), C.POINTER(C.c_uint32)]),
        "efg_csr_transpose": (i32, [u64, C.POINTER(C.c_uint64), C.POINTER(C.c_uint32), C.POINTER(C.c_uint64),
                                    C.POINTER(C.c_uint32)]),
        "efg_tree_count": (u32, [vp]),
        "efg_last_error": (C.c_char_p, []),
        "efg_version": (C.c_char_p, []),
        "efg_l2_pairs": (i32, [vp, u64, u32, u64, vp, vp, u64, vp, vp]),
        "efg_brute_force_knn": (i32, [vp, u64, u32, u64, vp, u64, u64, u32, i32, u64, vp, vp, vp]),
        "efg_brute_force_knn_noalloc": (i32, [vp, u64, u32, u64, vp, u64, u64, u32, i32, u64, vp, vp, vp]),
        "efg_brute_force_knn_fp32": (i32, [vp, u64, u32, u64, vp, u64, u64, u32, i32, u64, vp, vp, vp]),
        "efg_get_knn_stats": (i32, [vp]),
        "efg_brute_force_knn_split": (i32, [vp, u64, u32, u64, vp, u64, u64, u32, i32, u64, vp, vp, vp]),
        "efg_knn_search_batch": (i32, [vp, f32p, u64, u32, u64, vp, u32, C.POINTER(C.c_int32)]),
        "efg_knn_search_batch_device": (i32, [vp, vp, u64, u64, vp, C.POINTER(QueryParams), vp, vp, vp]),
        "efg_knn_search_seeded_device": (i32, [vp, vp, u64, u64, vp, C.POINTER(QueryParams), vp, u32, i32, vp, vp]),
        "efg_search_plan_create": (i32, [vp, u64, C.POINTER(QueryParams), f32p, u64, C.POINTER(vp)]),
        "efg_search_plan_submit": (i32, [vp, f32p, u64, u64, vp]),
        "efg_search_plan_collect": (i32, [vp, C.POINTER(C.c_int32)]),
        "efg_search_plan_run": (i32, [vp, f32p, u64, u64, vp, C.POINTER(C.c_int32)]),
        "efg_search_plan_threads": (i32, [vp]),
        "efg_search_plan_config": (i32, [vp, vp, vp, vp, vp, vp]),
        "efg_search_plan_destroy": (None, [vp]),
        "efg_learned_default_params": (None, [C.POINTER(LearnedParams)]),
        "efg_learned_create": (i32, [vp, C.POINTER(LearnedParams), C.POINTER(vp)]),
        "efg_learned_train": (i32, [vp, vp, u64, u64]),
        "efg_learned_predict_device": (i32, [vp, vp, u64, u64, C.c_float, vp, vp, vp]),
        "efg_learned_search_device": (i32, [vp, vp, u64, u64, u32, C.c_float, i32, vp, vp]),
        "efg_learned_get_stats": (i32, [vp, C.POINTER(LearnedStats)]),
        "efg_learned_num_params": (u64, [vp]),
        "efg_learned_get_weights": (i32, [vp, f32p]),
        "efg_learned_set_weights": (i32, [vp, f32p]),
        "efg_learned_get_norm": (i32, [vp, f32p, f32p]),
        "efg_learned_grad": (i32, [vp, vp, u32, u64, vp, vp, C.POINTER(C.c_double), f32p]),
        "efg_learned_clusters": (i32, [vp, vp, vp, vp]),
        "efg_learned_destroy": (None, [vp]),
        "efg_hash_create": (i32, [vp, vp, u32, u32, u32, C.POINTER(vp)]),
        "efg_hash_ball_size": (u64, [vp]),
        "efg_hash_seeds_device": (i32, [vp, vp, u64, u64, u32, vp, vp]),
        "efg_hash_search_device": (i32, [vp, vp, vp, u64, u64, vp, u64, u32, vp, vp]),
        "efg_hash_search": (i32, [vp, vp, f32p, u64, u32, u64, vp, u32, vp]),
        "efg_hash_destroy": (None, [vp]),
        "efg_nnd_init": (i32, [vp, C.POINTER(HostState)]),
        "efg_nnd_iterate": (i32, [vp, C.POINTER(HostState), u32, C.POINTER(C.c_uint64)]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _check(rc: int) -> None:
    if rc != EFG_OK:
        raise EfannaError(rc, lib().efg_last_error().decode())


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class Index:
    """FIndex<float> over the GPU implementation (efanna.hpp:9-75)."""

    def __init__(self, data: np.ndarray, params: IndexParams | None = None):
        data = np.ascontiguousarray(data, dtype=np.float32)
        if data.ndim != 2:
            raise ValueError("data must be 2-D (rows x dim)")
        self.n, self.dim = data.shape
        self.params = params or IndexParams()
        self._h = C.c_void_p()
        p = self.params.to_c()
        _check(lib().efg_index_create(_fp(data), self.n, self.dim, self.dim, C.byref(p), C.byref(self._h)))
        _live["index"].add(self)

    @classmethod
    def from_device(cls, ptr: int, n: int, dim: int, row_stride: int, params: IndexParams | None = None):
        self = cls.__new__(cls)
        self.n, self.dim = n, dim
        self.params = params or IndexParams()
        self._h = C.c_void_p()
        p = self.params.to_c()
        _check(lib().efg_index_create_device(C.c_void_p(ptr), n, dim, row_stride, C.byref(p), C.byref(self._h)))
        _live["index"].add(self)
        return self

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            # the plans, learned models and hash tables of this index use it until they are
            # destroyed (the library requires the index to outlive them): close them first
            for kind in ("learned", "plan", "hash"):
                for o in list(_live[kind]):
                    if getattr(o, "index", None) is self:
                        o.close()
            lib().efg_index_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # buildIndex / buildTrees
    def build_index(self) -> None:
        _check(lib().efg_build_graph(self._h))

    def build_trees(self, ntrees: int | None = None) -> None:
        if ntrees is None:
            _check(lib().efg_build_trees(self._h))
        else:
            _check(lib().efg_build_trees_count(self._h, ntrees))

    def build_stats(self) -> BuildStats:
        s = BuildStats()
        _check(lib().efg_get_build_stats(self._h, C.byref(s)))
        return s

    def search_stats(self) -> SearchStats:
        s = SearchStats()
        _check(lib().efg_get_search_stats(self._h, C.byref(s)))
        return s

    def set_search_params(self, epochs: int, init_num: int, extend_to: int, search_trees: int = 0,
                          search_lv: int = -1, search_method: int = 0) -> None:
        _check(lib().efg_set_search_params(self._h, epochs, init_num, extend_to, search_trees, search_lv,
                                           search_method))

    def set_search_precision(self, precision: str) -> None:
        """'fp32' (the reference's arithmetic), 'bf16' or 'fp8' (screening in that format, FP32 re-rank)."""
        code = {"fp32": 0, "bf16": 1, "fp8": 2}.get(precision)
        if code is None:
            raise ValueError("precision must be 'fp32', 'bf16' or 'fp8'")
        _check(lib().efg_set_search_precision(self._h, code))

    def set_build_precision(self, precision: str) -> None:
        """'fp32' (the reference's join arithmetic, the default) or 'bf16': the NN-descent join's pair
        distances as one Gram tile per node on the tensor cores (identical graph on byte data up to
        128 dimensions; hi + lo BF16 products for other data)."""
        code = {"fp32": 0, "bf16": 1}.get(precision)
        if code is None:
            raise ValueError("build precision must be 'fp32' or 'bf16'")
        _check(lib().efg_set_build_precision(self._h, code))

    def set_search_candidate_cap(self, cap: int) -> None:
        """Bound on the nnexp search's per-query candidate buffer (0: the worst case, the default)."""
        _check(lib().efg_set_search_candidate_cap(self._h, cap))

    def screen_distances_device(self, precision: str, q_ptr: int, nq: int, row_stride: int, ids_ptr: int, m: int,
                                out_ptr: int, stream: int = 0):
        code = {"fp32": 0, "bf16": 1, "fp8": 2}[precision]
        _check(lib().efg_screen_distances(self._h, code, C.c_void_p(q_ptr), nq, row_stride, C.c_void_p(ids_ptr), m,
                                          C.c_void_p(out_ptr), C.c_void_p(stream)))

    def knn_search(self, k: int, queries: np.ndarray) -> np.ndarray:
        q = np.ascontiguousarray(queries, dtype=np.float32)
        out = np.zeros((q.shape[0], k), dtype=np.int32)
        _check(lib().efg_knn_search(self._h, _fp(q), q.shape[0], q.shape[1], q.shape[1], k,
                                    out.ctypes.data_as(C.POINTER(C.c_int32))))
        return out

    def knn_search_batch(self, queries: np.ndarray, params, k_max: int) -> np.ndarray:
        """Per-query (epochs, pool, extend, k) rows; returns nq x k_max ids, -1 past each k."""
        q = np.ascontiguousarray(queries, dtype=np.float32)
        p = query_params(params)
        out = np.zeros((q.shape[0], k_max), dtype=np.int32)
        _check(lib().efg_knn_search_batch(self._h, _fp(q), q.shape[0], q.shape[1], q.shape[1],
                                          C.c_void_p(p.ctypes.data), k_max,
                                          out.ctypes.data_as(C.POINTER(C.c_int32))))
        return out

    def knn_search_batch_device(self, q_ptr: int, nq: int, row_stride: int, params_ptr: int, limits, out_ptr: int,
                                nq_ptr: int = 0, stream: int = 0):
        lim = QueryParams(*[int(v) for v in limits])
        _check(lib().efg_knn_search_batch_device(self._h, C.c_void_p(q_ptr), nq, row_stride, C.c_void_p(params_ptr),
                                                 C.byref(lim), C.c_void_p(out_ptr), C.c_void_p(nq_ptr or None),
                                                 C.c_void_p(stream)))

    def knn_search_seeded_device(self, q_ptr: int, nq: int, row_stride: int, params_ptr: int, limits, seeds_ptr: int,
                                 seeds_per_query: int, out_ptr: int, stream: int = 0, use_trees: bool = True):
        lim = QueryParams(*[int(v) for v in limits])
        _check(lib().efg_knn_search_seeded_device(self._h, C.c_void_p(q_ptr), nq, row_stride,
                                                  C.c_void_p(params_ptr or None), C.byref(lim),
                                                  C.c_void_p(seeds_ptr), seeds_per_query, int(use_trees),
                                                  C.c_void_p(out_ptr), C.c_void_p(stream)))

    def search_plan(self, capacity: int, limits, calib: np.ndarray | None = None) -> "SearchPlan":
        return SearchPlan(self, capacity, limits, calib)

    def knn_search_device(self, k: int, q_ptr: int, nq: int, row_stride: int, out_ptr: int, stream: int = 0):
        _check(lib().efg_knn_search_device(self._h, C.c_void_p(q_ptr), nq, row_stride, k, C.c_void_p(out_ptr),
                                           C.c_void_p(stream)))

    # files
    def save_graph(self, path: str): _check(lib().efg_save_graph(self._h, path.encode()))
    def load_graph(self, path: str): _check(lib().efg_load_graph(self._h, path.encode()))
    def save_trees(self, path: str): _check(lib().efg_save_trees(self._h, path.encode()))
    def load_trees(self, path: str): _check(lib().efg_load_trees(self._h, path.encode()))
    def save_index(self, path: str): _check(lib().efg_save_index(self._h, path.encode()))
    def load_index(self, path: str): _check(lib().efg_load_index(self._h, path.encode()))
    def save_results(self, path: str): _check(lib().efg_save_results(self._h, path.encode()))

    def graph_size(self) -> int:
        return int(lib().efg_graph_size(self._h))

    def graph_row(self, row: int) -> list:
        n = lib().efg_graph_row(self._h, row, None, 0)
        if n < 0:
            _check(EFG_ERR_ARG)
        buf = (C.c_uint32 * max(1, n))()
        lib().efg_graph_row(self._h, row, buf, n)
        return list(buf[:n])

    def graph_csr(self):
        nnz = C.c_uint64()
        _check(lib().efg_graph_csr(self._h, None, None, C.byref(nnz)))
        ptr = np.zeros(self.graph_size() + 1, np.uint64)
        ids = np.zeros(max(1, nnz.value), np.uint32)
        _check(lib().efg_graph_csr(self._h, ptr.ctypes.data_as(C.POINTER(C.c_uint64)),
                                   ids.ctypes.data_as(C.POINTER(C.c_uint32)), None))
        return ptr, ids[:nnz.value]

    def graph_csc(self):
        """The graph in compressed-column form (the MATLAB front end's getGraphMat): col_ptr (n + 1) and
        row_ids, column j holding the nodes whose rows list j, ascending."""
        n = self.graph_size()
        nnz = C.c_uint64()
        _check(lib().efg_graph_csr(self._h, None, None, C.byref(nnz)))
        col_ptr = np.zeros(n + 1, np.uint64)
        row_ids = np.zeros(max(1, nnz.value), np.uint32)
        _check(lib().efg_graph_csc(self._h, col_ptr.ctypes.data_as(C.POINTER(C.c_uint64)),
                                   row_ids.ctypes.data_as(C.POINTER(C.c_uint32))))
        return col_ptr, row_ids[:nnz.value]

    def graph(self) -> np.ndarray:
        """Fixed-degree graph as an (n, K) array."""
        ptr, ids = self.graph_csr()
        return ids.reshape(self.graph_size(), -1)

    def tree_count(self) -> int:
        return int(lib().efg_tree_count(self._h))

    # state-level NN-descent (parity tests)
    def nnd_init(self, st) -> None:
        hs = _host_state(st)
        _check(lib().efg_nnd_init(self._h, C.byref(hs)))

    def nnd_iterate(self, st, it: int) -> int:
        hs = _host_state(st)
        pairs = C.c_uint64()
        _check(lib().efg_nnd_iterate(self._h, C.byref(hs), it, C.byref(pairs)))
        return int(pairs.value)


class SearchPlan:
    """A captured batched search (efg_search_plan): run(queries, params) -> nq x limits.k ids."""

    def __init__(self, index: "Index", capacity: int, limits, calib: np.ndarray | None = None):
        self.index = index
        self.limits = QueryParams(*[int(v) for v in limits])
        h = C.c_void_p()
        cq = None if calib is None else np.ascontiguousarray(calib, dtype=np.float32)
        _check(lib().efg_search_plan_create(index._h, capacity, C.byref(self.limits),
                                            None if cq is None else _fp(cq), 0 if cq is None else cq.shape[0],
                                            C.byref(h)))
        self._h = h
        _live["plan"].add(self)

    @property
    def threads(self) -> int:
        return lib().efg_search_plan_threads(self._h)

    @property
    def config(self) -> dict:
        """The launch the autotuner chose: threads, ctas_per_sm (0: as many as fit), ht_pct (shared
        visited-set size in percent of the default), variants timed, tuned_ms."""
        v = [C.c_int32() for _ in range(4)]
        ms = C.c_double()
        _check(lib().efg_search_plan_config(self._h, *[C.byref(x) for x in v], C.byref(ms)))
        return {"threads": v[0].value, "ctas_per_sm": v[1].value, "ht_pct": v[2].value, "variants": v[3].value,
                "tuned_ms": round(ms.value, 3)}

    def run(self, queries: np.ndarray, params, out: np.ndarray | None = None) -> np.ndarray:
        q = np.ascontiguousarray(queries, dtype=np.float32)
        p = query_params(params)
        if out is None:
            out = np.zeros((q.shape[0], self.limits.k), dtype=np.int32)
        _check(lib().efg_search_plan_run(self._h, _fp(q), q.shape[0], q.shape[1], C.c_void_p(p.ctypes.data),
                                         out.ctypes.data_as(C.POINTER(C.c_int32))))
        return out

    def submit(self, queries: np.ndarray, params) -> int:
        """Queues a batch without waiting (the rows are staged before this returns); collect()
        writes its ids.  Returns the batch size."""
        q = np.ascontiguousarray(queries, dtype=np.float32)
        p = query_params(params)
        _check(lib().efg_search_plan_submit(self._h, _fp(q), q.shape[0], q.shape[1], C.c_void_p(p.ctypes.data)))
        self._pending = q.shape[0]
        return q.shape[0]

    def collect(self, out: np.ndarray | None = None) -> np.ndarray:
        n = getattr(self, "_pending", 0)
        if out is None:
            out = np.zeros((n, self.limits.k), dtype=np.int32)
        _check(lib().efg_search_plan_collect(self._h, out.ctypes.data_as(C.POINTER(C.c_int32))))
        self._pending = 0
        return out[:n]

    def close(self):
        if self._h:
            lib().efg_search_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Learned:
    """The learned form (efg_learned): k-means entry clusters + an MLP trained on search traces.
    ``rungs`` is a list of (epochs, pool, extend) settings in ascending cost."""

    def __init__(self, index: "Index", clusters=1024, entries_per_cluster=16, entry_clusters=8, hidden=256,
                 rungs=None, target=0.9, train_epochs=8, batch=1024, lr=1e-3, kmeans_iters=10,
                 kmeans_sample=100000, seed=1998, trace_reference=None):
        p = LearnedParams()
        lib().efg_learned_default_params(C.byref(p))
        p.clusters, p.entries_per_cluster, p.entry_clusters, p.hidden = clusters, entries_per_cluster, \
            entry_clusters, hidden
        p.target, p.train_epochs, p.batch, p.lr = target, train_epochs, batch, lr
        p.kmeans_iters, p.kmeans_sample, p.seed = kmeans_iters, kmeans_sample, seed
        if trace_reference is not None:  # (epochs, pool, extend): traces scored against that plain search
            p.trace_reference = QueryParams(int(trace_reference[0]), int(trace_reference[1]),
                                            int(trace_reference[2]), 10)
        if rungs is not None:
            p.rungs = len(rungs)
            for i, r in enumerate(rungs):
                p.rung[i] = QueryParams(int(r[0]), int(r[1]), int(r[2]), 10)
        self.params = p
        self.index = index
        h = C.c_void_p()
        _check(lib().efg_learned_create(index._h, C.byref(p), C.byref(h)))
        self._h = h
        _live["learned"].add(self)

    @property
    def rungs(self):
        return [(self.params.rung[i].epochs, self.params.rung[i].init_num, self.params.rung[i].extend_to)
                for i in range(self.params.rungs)]

    def train_device(self, q_ptr: int, n: int, row_stride: int):
        _check(lib().efg_learned_train(self._h, C.c_void_p(q_ptr), n, row_stride))

    def predict_device(self, q_ptr: int, nq: int, row_stride: int, clusters_ptr: int, rung_ptr: int, stream: int = 0,
                       coverage: float = 0.0):
        _check(lib().efg_learned_predict_device(self._h, C.c_void_p(q_ptr), nq, row_stride, coverage,
                                                C.c_void_p(clusters_ptr or None), C.c_void_p(rung_ptr),
                                                C.c_void_p(stream)))

    def search_device(self, q_ptr: int, nq: int, row_stride: int, k: int, out_ptr: int, rung_bias: int = 0,
                      stream: int = 0, coverage: float = 0.0):
        _check(lib().efg_learned_search_device(self._h, C.c_void_p(q_ptr), nq, row_stride, k, coverage, rung_bias,
                                               C.c_void_p(out_ptr), C.c_void_p(stream)))

    def stats(self) -> LearnedStats:
        st = LearnedStats()
        _check(lib().efg_learned_get_stats(self._h, C.byref(st)))
        return st

    def num_params(self) -> int:
        return int(lib().efg_learned_num_params(self._h))

    def weights(self) -> np.ndarray:
        w = np.zeros(self.num_params(), np.float32)
        _check(lib().efg_learned_get_weights(self._h, _fp(w)))
        return w

    def set_weights(self, w: np.ndarray):
        w = np.ascontiguousarray(w, np.float32)
        _check(lib().efg_learned_set_weights(self._h, _fp(w)))

    def norm(self):
        d = self.index.dim
        mean, istd = np.zeros(d, np.float32), np.zeros(d, np.float32)
        _check(lib().efg_learned_get_norm(self._h, _fp(mean), _fp(istd)))
        return mean, istd

    def grad_device(self, x_ptr: int, B: int, row_stride: int, tc_ptr: int, tl_ptr: int):
        g = np.zeros(self.num_params(), np.float32)
        loss = C.c_double()
        _check(lib().efg_learned_grad(self._h, C.c_void_p(x_ptr), B, row_stride, C.c_void_p(tc_ptr),
                                      C.c_void_p(tl_ptr), C.byref(loss), _fp(g)))
        return loss.value, g

    def clusters(self):
        n, C_, m = self.index.n, self.params.clusters, max(self.params.entries_per_cluster, 1)
        a = np.zeros(n, np.int32)
        e = np.zeros((C_, m), np.uint32)
        c = np.zeros(C_, np.uint32)
        _check(lib().efg_learned_clusters(self._h, C.c_void_p(a.ctypes.data), C.c_void_p(e.ctypes.data),
                                          C.c_void_p(c.ctypes.data)))
        return a, e, c

    def close(self):
        if self._h:
            lib().efg_learned_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class HashTables:
    """The hashing initialiser's tables (efg_hash) over an Index's base, for the hashing-seeded
    search (HASHINGIndex with search method 1, algorithm/hashing_index.hpp:1087-1200).  ``codes`` is
    tables x n codes of ``code_bits`` bits; the search uses the index's graph and its search
    parameters (epochs, pool, extend), and no trees."""

    def __init__(self, index: "Index", codes: np.ndarray, code_bits: int, radius: int):
        c = np.ascontiguousarray(codes, dtype=np.uint64)
        if c.ndim != 2 or c.shape[1] != index.n:
            raise ValueError("codes must be tables x n")
        self.index, self.tables, self.code_bits, self.radius = index, c.shape[0], code_bits, radius
        h = C.c_void_p()
        _check(lib().efg_hash_create(index._h, C.c_void_p(c.ctypes.data), c.shape[0], code_bits, radius,
                                     C.byref(h)))
        self._h = h
        _live["hash"].add(self)

    @property
    def ball_size(self) -> int:
        return int(lib().efg_hash_ball_size(self._h))

    def search(self, k: int, queries: np.ndarray, qcodes: np.ndarray) -> np.ndarray:
        q = np.ascontiguousarray(queries, dtype=np.float32)
        qc = np.ascontiguousarray(qcodes, dtype=np.uint64)
        if qc.shape != (self.tables, q.shape[0]):
            raise ValueError("qcodes must be tables x nq")
        out = np.zeros((q.shape[0], k), dtype=np.int32)
        _check(lib().efg_hash_search(self.index._h, self._h, _fp(q), q.shape[0], q.shape[1], q.shape[1],
                                     C.c_void_p(qc.ctypes.data), k, C.c_void_p(out.ctypes.data)))
        return out

    def search_device(self, q_ptr: int, nq: int, row_stride: int, qcodes_ptr: int, qcode_stride: int, k: int,
                      out_ptr: int, stream: int = 0):
        _check(lib().efg_hash_search_device(self.index._h, self._h, C.c_void_p(q_ptr), nq, row_stride,
                                            C.c_void_p(qcodes_ptr), qcode_stride, k, C.c_void_p(out_ptr),
                                            C.c_void_p(stream)))

    def seeds_device(self, qcodes_ptr: int, qcode_stride: int, nq: int, seeds_per_query: int, out_ptr: int,
                     stream: int = 0):
        _check(lib().efg_hash_seeds_device(self._h, C.c_void_p(qcodes_ptr), qcode_stride, nq, seeds_per_query,
                                           C.c_void_p(out_ptr), C.c_void_p(stream)))

    def close(self):
        if self._h:
            lib().efg_hash_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _host_state(st) -> HostState:
    """Wraps an object with the state arrays (n, Lcap, cap, pool_dist, ...) of one layout."""
    def p(a, t):
        assert a.flags.c_contiguous
        return a.ctypes.data_as(C.POINTER(t))
    return HostState(st.n, st.Lcap, st.cap, p(st.pool_dist, C.c_float), p(st.pool_id, C.c_uint32),
                     p(st.pool_flag, C.c_uint8), p(st.L, C.c_uint32), p(st.Range, C.c_uint32),
                     p(st.radius, C.c_float), p(st.radiusM, C.c_float), p(st.found, C.c_uint8),
                     p(st.new_ids, C.c_uint32), p(st.new_cnt, C.c_uint32), p(st.old_ids, C.c_uint32),
                     p(st.old_cnt, C.c_uint32))


def l2_pairs_device(base_ptr: int, n: int, dim: int, row_stride: int, a_ptr: int, b_ptr: int, m: int,
                    out_ptr: int, stream: int = 0) -> None:
    _check(lib().efg_l2_pairs(C.c_void_p(base_ptr), n, dim, row_stride, C.c_void_p(a_ptr), C.c_void_p(b_ptr), m,
                              C.c_void_p(out_ptr), C.c_void_p(stream)))


class KnnStats(C.Structure):
    _fields_ = [("convert_ms", C.c_double), ("bound_ms", C.c_double), ("screen_ms", C.c_double),
                ("merge_ms", C.c_double), ("screen_flops", C.c_double), ("tile_flops", C.c_double),
                ("terms", C.c_uint32), ("stages", C.c_uint32), ("nchunks", C.c_uint32), ("ctas", C.c_uint32),
                ("sample_rows", C.c_uint32)]


def knn_stats() -> KnnStats:
    """Timing of this thread's last tensor-core exact k-NN call."""
    st = KnnStats()
    _check(lib().efg_get_knn_stats(C.byref(st)))
    return st


def csr_transpose(row_ptr: np.ndarray, ids: np.ndarray, n: int):
    """efg_csr_transpose: the compressed-column form of a CSR graph over n nodes (host arrays)."""
    row_ptr = np.ascontiguousarray(row_ptr, np.uint64)
    ids = np.ascontiguousarray(ids, np.uint32)
    col_ptr = np.zeros(n + 1, np.uint64)
    row_ids = np.zeros(max(1, int(row_ptr[n])), np.uint32)
    _check(lib().efg_csr_transpose(n, row_ptr.ctypes.data_as(C.POINTER(C.c_uint64)),
                                   ids.ctypes.data_as(C.POINTER(C.c_uint32)),
                                   col_ptr.ctypes.data_as(C.POINTER(C.c_uint64)),
                                   row_ids.ctypes.data_as(C.POINTER(C.c_uint32))))
    return col_ptr, row_ids[:int(row_ptr[n])]


def brute_force_knn_device(base_ptr: int, n: int, dim: int, row_stride: int, q_ptr: int, nq: int, q_stride: int,
                           k: int, ids_ptr: int, dists_ptr: int = 0, exclude_self: bool = False, first_row: int = 0,
                           stream: int = 0, screening: str = "auto") -> None:
    """Exact k-NN (efg_brute_force_knn).  screening: 'auto' (tensor cores for k <= 104), 'fp32'
    (the FP32 CUDA-core kernel) or 'split' (tensor cores with the hi + lo split forced)."""
    fn = {"auto": "efg_brute_force_knn", "fp32": "efg_brute_force_knn_fp32",
          "split": "efg_brute_force_knn_split"}[screening]
    _check(getattr(lib(), fn)(C.c_void_p(base_ptr), n, dim, row_stride, C.c_void_p(q_ptr), nq, q_stride, k,
                              int(exclude_self), first_row, C.c_void_p(ids_ptr), C.c_void_p(dists_ptr or None),
                              C.c_void_p(stream)))


def brute_force_knn_device_noalloc(base_ptr: int, n: int, dim: int, row_stride: int, q_ptr: int, nq: int,
                                   q_stride: int, k: int, ids_ptr: int, dists_ptr: int = 0, exclude_self: bool = False,
                                   first_row: int = 0, stream: int = 0) -> None:
    """efg_brute_force_knn_noalloc: the same results with no device allocation (fixed built-in scratch)."""
    _check(lib().efg_brute_force_knn_noalloc(C.c_void_p(base_ptr), n, dim, row_stride, C.c_void_p(q_ptr), nq,
                                             q_stride, k, int(exclude_self), first_row, C.c_void_p(ids_ptr),
                                             C.c_void_p(dists_ptr or None), C.c_void_p(stream)))


def version() -> str:
    return lib().efg_version().decode()
