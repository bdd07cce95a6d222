"""Readers and writers for the reference's vector and index-side files.

* fvecs / ivecs: each row is an int32 ``d`` followed by ``d`` float32 / int32 values
  (samples/efanna_index_buildgraph.cc:10-29, samples/evaluate.cc:6-22).
* graph: per row a uint32 ``k`` followed by ``k`` uint32 ids, i.e. ivecs
  (algorithm/kdtreeub_index.hpp:243-312); rows may have different ``k``.
* results: ivecs (algorithm/base_index.hpp:136-151).
"""
from __future__ import annotations

import numpy as np


def write_vecs(path: str, x: np.ndarray) -> None:
    x = np.ascontiguousarray(x)
    n, d = x.shape
    rows = np.empty((n, d + 1), dtype=np.int32)
    rows[:, 0] = d
    rows[:, 1:] = x.view(np.int32) if x.dtype.itemsize == 4 else x.astype(np.int32)
    rows.tofile(path)


def write_fvecs(path: str, x: np.ndarray) -> None:
    write_vecs(path, np.ascontiguousarray(x, dtype=np.float32))


def write_ivecs(path: str, x: np.ndarray) -> None:
    write_vecs(path, np.ascontiguousarray(x, dtype=np.int32))


def read_ivecs(path: str) -> np.ndarray:
    raw = np.fromfile(path, dtype=np.int32)
    if raw.size == 0:
        return np.zeros((0, 0), dtype=np.int32)
    d = int(raw[0])
    return raw.reshape(-1, d + 1)[:, 1:].copy()


def read_fvecs(path: str) -> np.ndarray:
    return read_ivecs(path).view(np.float32)


def read_graph_csr(path: str):
    """Variable-degree graph file -> (row_ptr uint64[n+1], ids uint32[nnz])."""
    raw = np.fromfile(path, dtype=np.uint32)
    ptr = [0]
    ids = []
    i = 0
    while i < raw.size:
        k = int(raw[i])
        ids.append(raw[i + 1:i + 1 + k])
        ptr.append(ptr[-1] + k)
        i += k + 1
    cat = np.concatenate(ids) if ids else np.zeros(0, np.uint32)
    return np.asarray(ptr, dtype=np.uint64), cat.astype(np.uint32)
