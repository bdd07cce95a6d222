"""efg_brute_force_knn_noalloc: the brute-force k-NN for callers that cannot let the library
allocate device memory during a call (their GPU memory belongs to another allocator, or the call
sits in a loop that must not pay for an allocation).  Called through the C ABI, it must return
what the allocating entry point returns, on consecutive calls that share its built-in scratch.
Collected last so that a failure here stops a -x run only after every other test has run."""
import ctypes as C

import numpy as np
import pytest

from efanna_gb300 import datasets

pytestmark = pytest.mark.gpu


def _run(efg, fn, X, n, Q, nq, k, exclude):
    import torch
    ids = torch.full((nq, k), -7, dtype=torch.int32, device="cuda")
    dist = torch.full((nq, k), -1.0, dtype=torch.float32, device="cuda")
    rc = fn(C.c_void_p(X.data_ptr()), n, X.shape[1], X.shape[1], C.c_void_p(Q.data_ptr()), nq, Q.shape[1], k,
            int(exclude), 0, C.c_void_p(ids.data_ptr()), C.c_void_p(dist.data_ptr()), None)
    torch.cuda.synchronize()
    assert rc == 0, efg.lib().efg_last_error()
    return ids.cpu().numpy(), dist.cpu().numpy()


def test_noalloc_matches_allocating_entry_point_on_consecutive_calls(efg):
    torch = pytest.importorskip("torch")
    lib = efg.lib()
    x = datasets.mixture_u8(30000, 128, seed=21)
    X = torch.from_numpy(x).cuda()
    cases = [  # two calls in a row with different shapes, then a repeat of the first
        (torch.from_numpy(datasets.mixture_u8(700, 128, seed=21, queries=True)).cuda(), 10, False),
        (X[:500].contiguous(), 32, True),
        (torch.from_numpy(datasets.mixture_u8(700, 128, seed=21, queries=True)).cuda(), 10, False),
    ]
    for Q, k, exclude in cases:
        want = _run(efg, lib.efg_brute_force_knn, X, 30000, Q, Q.shape[0], k, exclude)
        got = _run(efg, lib.efg_brute_force_knn_noalloc, X, 30000, Q, Q.shape[0], k, exclude)
        assert np.array_equal(got[0], want[0])
        assert np.array_equal(got[1], want[1])


def test_noalloc_float_data_and_size_limit(efg):
    torch = pytest.importorskip("torch")
    lib = efg.lib()
    x = datasets.mixture_unit(8000, 64, block=16, seed=5)
    X = torch.from_numpy(x).cuda()
    Q = torch.from_numpy(datasets.mixture_unit(300, 64, block=16, seed=5, queries=True)).cuda()
    want = _run(efg, lib.efg_brute_force_knn, X, 8000, Q, 300, 20, False)
    got = _run(efg, lib.efg_brute_force_knn_noalloc, X, 8000, Q, 300, 20, False)
    assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])
    # nq * (k + 16) beyond the built-in scratch is refused with a clear error
    big = torch.zeros((20000, 64), dtype=torch.float32, device="cuda")
    ids = torch.zeros((20000, 256), dtype=torch.int32, device="cuda")
    rc = lib.efg_brute_force_knn_noalloc(C.c_void_p(X.data_ptr()), 8000, 64, 64, C.c_void_p(big.data_ptr()), 20000,
                                         64, 256, 0, 0, C.c_void_p(ids.data_ptr()), None, None)
    assert rc == efg.EFG_ERR_ARG
    assert b"scratch" in lib.efg_last_error()


def test_noalloc_strides_exclude_self_and_stream(efg):
    """Padded rows (dim 33 in rows of 36 floats, queries in rows of 40), exclude_self with a
    non-zero first row, and a call on a non-default stream: the same ids and distances as the
    allocating entry point, whose smaller chunk count the fixed scratch may force."""
    torch = pytest.importorskip("torch")
    lib = efg.lib()
    x = datasets.mixture_u8(6000, 33, seed=12)
    xp = np.zeros((6000, 36), np.float32)
    xp[:, :33] = x
    first = 2500
    qp = np.zeros((700, 40), np.float32)
    qp[:, :33] = x[first:first + 700]
    X, Q = torch.from_numpy(xp).cuda(), torch.from_numpy(qp).cuda()
    s = torch.cuda.Stream()
    out = {}
    for name, stream in (("efg_brute_force_knn", None), ("efg_brute_force_knn_noalloc", s.cuda_stream)):
        ids = torch.full((700, 16), -7, dtype=torch.int32, device="cuda")
        dist = torch.full((700, 16), -1.0, dtype=torch.float32, device="cuda")
        rc = getattr(lib, name)(C.c_void_p(X.data_ptr()), 6000, 33, 36, C.c_void_p(Q.data_ptr()), 700, 40, 16, 1, first,
                                C.c_void_p(ids.data_ptr()), C.c_void_p(dist.data_ptr()),
                                C.c_void_p(stream) if stream else None)
        torch.cuda.synchronize()
        assert rc == 0, lib.efg_last_error()
        out[name] = (ids.cpu().numpy(), dist.cpu().numpy())
    want, got = out["efg_brute_force_knn"], out["efg_brute_force_knn_noalloc"]
    assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])
    assert not np.any(got[0] == (first + np.arange(700))[:, None])
