"""Readers and writers for the reference's vector and index-side files.

* fvecs / ivecs: each row is an int32 ``d`` followed by ``d`` float32 / int32 values
  (samples/efanna_index_buildgraph.cc:10-29, samples/evaluate.cc:6-22).
* graph: per row a uint32 ``k`` followed by ``k`` uint32 ids, i.e. ivecs
  (algorithm/kdtreeub_index.hpp:243-312); rows may have different ``k``.
* results: ivecs (algorithm/base_index.hpp:136-151).
* hash codes: one file ``<prefix>_<t>`` per table t = 1..tables, holding int32 1, int32 code length,
  int32 count, then the codes as uint32 (code length <= 32) or uint64 (algorithm/hashing_index.hpp:
  206-300, LoadCode32 / LoadCode64).
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


def write_codes(prefix: str, codes: np.ndarray, code_len: int) -> None:
    """tables x n codes -> the hashing initialiser's code files ``<prefix>_1`` ... ``<prefix>_<tables>``."""
    codes = np.asarray(codes, dtype=np.uint64)
    wide = code_len > 32
    for t in range(codes.shape[0]):
        with open("%s_%d" % (prefix, t + 1), "wb") as f:
            np.array([1, code_len, codes.shape[1]], np.int32).tofile(f)
            codes[t].astype(np.uint64 if wide else np.uint32).tofile(f)


def read_codes(prefix: str, tables: int, code_len: int, shift: int = 0):
    """The code files of ``tables`` tables -> (tables x n uint64 codes, code bits).  Like the
    reference, ``code_len`` (the index parameter) picks 32- or 64-bit words and bounds the shifted
    codes (a code of more than ``code_len - shift`` bits is an error), every code is shifted right
    by ``shift``, and the file's own code length minus ``shift`` is the length the Hamming ball
    uses."""
    if code_len > 64:
        raise ValueError("code length not supported: at most 64 bits")
    out, bits = [], None
    for t in range(tables):
        raw = np.fromfile("%s_%d" % (prefix, t + 1), dtype=np.uint8)
        head = raw[:12].view(np.int32)
        if raw.size < 12 or head[0] != 1:
            raise ValueError("code file %s_%d: bad header" % (prefix, t + 1))
        file_len, num = int(head[1]), int(head[2])
        word = np.uint64 if code_len > 32 else np.uint32
        body = raw[12:12 + num * np.dtype(word).itemsize]
        if body.size != num * np.dtype(word).itemsize:
            raise ValueError("code file %s_%d: truncated" % (prefix, t + 1))
        c = body.view(word).astype(np.uint64) >> np.uint64(shift)
        b = file_len - shift
        if b <= 0 or b > 64:
            raise ValueError("code file %s_%d: code length %d with shift %d" % (prefix, t + 1, file_len, shift))
        lim = code_len - shift
        if lim <= 0 or (lim < 64 and np.any(c >> np.uint64(lim))):
            raise ValueError("code file %s_%d: a code exceeds %d bits" % (prefix, t + 1, lim))
        if bits is not None and b != bits:
            raise ValueError("code files disagree on the code length")
        bits = b
        out.append(c)
    return np.stack(out), bits
