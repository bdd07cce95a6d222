"""The exact k-NN with its screening on the tensor cores (tcgen05 BF16 Gram tiles, FP32
accumulation, then the FP64 re-rank) against the FP32 CUDA-core screening and against numpy.

On byte-valued data BF16 holds every value and every FP32 partial sum of the Gram form is an
exact integer, so both screenings keep the same survivors and the results must be bit-identical.
On general float data the tensor-core path splits each value into hi + lo BF16 parts; the ids
after the FP64 re-rank must still be the exact ones."""
import numpy as np
import pytest

from efanna_gb300 import datasets

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _knn(efg, x, q, k, screening, exclude=False, first_row=0, stride=None, qstride=None, stream=0):
    n, d = x.shape
    ld = stride or (d + 3) // 4 * 4   # rows start on 16-byte boundaries
    qld = qstride or (d + 3) // 4 * 4
    xp = np.zeros((n, ld), np.float32)
    xp[:, :d] = x
    qp = np.zeros((q.shape[0], qld), np.float32)
    qp[:, :d] = q
    X, Q = torch.from_numpy(xp).cuda(), torch.from_numpy(qp).cuda()
    ids = torch.full((q.shape[0], k), -7, dtype=torch.int32, device="cuda")
    dist = torch.full((q.shape[0], k), -1.0, dtype=torch.float32, device="cuda")
    efg.brute_force_knn_device(X.data_ptr(), n, d, ld, Q.data_ptr(), q.shape[0], qld, k, ids.data_ptr(),
                               dist.data_ptr(), exclude_self=exclude, first_row=first_row, stream=stream,
                               screening=screening)
    torch.cuda.synchronize()
    return ids.cpu().numpy(), dist.cpu().numpy()


def _numpy_exact(x, q, k, exclude_rows=None):
    xd, qd = x.astype(np.float64), q.astype(np.float64)
    D = ((qd[:, None, :] - xd[None, :, :]) ** 2).sum(2)
    if exclude_rows is not None:
        D[np.arange(len(q)), exclude_rows] = np.inf
    order = np.lexsort((np.broadcast_to(np.arange(len(x)), D.shape), D), axis=1)[:, :k]
    return order.astype(np.int32), np.take_along_axis(D, order, 1)


@pytest.mark.parametrize("d", [1, 3, 32, 64, 100, 128, 200, 960])
@pytest.mark.parametrize("k", [1, 10, 100])
def test_tensor_core_equals_fp32_on_byte_data(efg, d, k):
    n, nq = 3000 + 77, 300
    x = datasets.mixture_u8(n, d, seed=d) if d >= 8 else np.random.default_rng(d).integers(0, 256, (n, d)).astype(
        np.float32)
    q = datasets.mixture_u8(nq, d, seed=d, queries=True) if d >= 8 else \
        np.random.default_rng(d + 1).integers(0, 256, (nq, d)).astype(np.float32)
    tc = _knn(efg, x, q, k, "auto")
    f32 = _knn(efg, x, q, k, "fp32")
    assert np.array_equal(tc[0], f32[0]) and np.array_equal(tc[1], f32[1])
    if d <= 128:
        ref_ids, ref_d = _numpy_exact(x, q, k)
        assert np.array_equal(tc[0], ref_ids)
        assert np.array_equal(tc[1], ref_d.astype(np.float32))


def test_split_form_on_byte_data_equals_plain(efg):
    x = datasets.mixture_u8(5000, 128, seed=3)
    q = datasets.mixture_u8(257, 128, seed=3, queries=True)
    plain = _knn(efg, x, q, 10, "auto")
    split = _knn(efg, x, q, 10, "split")
    assert np.array_equal(plain[0], split[0]) and np.array_equal(plain[1], split[1])


def test_exclude_self_strides_and_stream(efg):
    """exclude_self with a non-zero first row, padded row strides (dim 33 in rows of 36 floats) and
    a call on a non-default stream: identical to the FP32 screening and to numpy."""
    x = datasets.mixture_u8(4000, 33, seed=8)
    rows = np.arange(1500, 1500 + 400)
    s = torch.cuda.Stream()
    tc = _knn(efg, x, x[rows], 12, "auto", exclude=True, first_row=1500, stride=36, qstride=40,
              stream=s.cuda_stream)
    f32 = _knn(efg, x, x[rows], 12, "fp32", exclude=True, first_row=1500, stride=36, qstride=40)
    ref_ids, _ = _numpy_exact(x, x[rows], 12, exclude_rows=rows)
    assert np.array_equal(tc[0], f32[0]) and np.array_equal(tc[1], f32[1])
    assert np.array_equal(tc[0], ref_ids)
    assert not np.any(tc[0] == rows[:, None])


@pytest.mark.parametrize("gen,d", [("unit", 960), ("unit", 128), ("gauss", 96)])
def test_tensor_core_split_ids_exact_on_float_data(efg, gen, d):
    """Float data (the d = 960 unit-block generator; a Gaussian at d = 96): the split BF16 screening
    keeps the true neighbours among its survivors, so the ids after the FP64 re-rank equal numpy's
    exact FP64 order, and so do the FP32 screening's."""
    n, nq, k = 6000, 200, 100 if d == 960 else 10
    if gen == "unit":
        x = datasets.mixture_unit(n, d, block=16, seed=2)
        q = datasets.mixture_unit(nq, d, block=16, seed=2, queries=True)
    else:
        rng = np.random.default_rng(4)
        x = rng.standard_normal((n, d)).astype(np.float32)
        q = rng.standard_normal((nq, d)).astype(np.float32)
    tc = _knn(efg, x, q, k, "auto")
    ref_ids, ref_d = _numpy_exact(x, q, k)
    f32 = _knn(efg, x, q, k, "fp32")
    assert np.array_equal(tc[0], ref_ids)
    assert np.array_equal(tc[0], f32[0])
    assert np.allclose(tc[1], ref_d, rtol=1e-6, atol=0)


def test_tensor_core_full_size_equals_fp32(efg):
    """The benchmark's ground truth: 1M x 128 byte-valued base, 2,000 held-out queries, k = 10."""
    x = datasets.mixture_u8(1_000_000, 128, seed=0)
    q = datasets.mixture_u8(2000, 128, seed=0, queries=True)
    X, Q = torch.from_numpy(x).cuda(), torch.from_numpy(q).cuda()
    out = {}
    for screening in ("auto", "fp32"):
        ids = torch.zeros((2000, 10), dtype=torch.int32, device="cuda")
        dist = torch.zeros((2000, 10), dtype=torch.float32, device="cuda")
        efg.brute_force_knn_device(X.data_ptr(), 1_000_000, 128, 128, Q.data_ptr(), 2000, 128, 10, ids.data_ptr(),
                                   dist.data_ptr(), screening=screening)
        torch.cuda.synchronize()
        out[screening] = (ids.cpu().numpy(), dist.cpu().numpy())
    assert np.array_equal(out["auto"][0], out["fp32"][0])
    assert np.array_equal(out["auto"][1], out["fp32"][1])
