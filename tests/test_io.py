import numpy as np

from efanna_gb300 import datasets, io


def test_vecs_roundtrip(tmp_path):
    x = datasets.mixture_u8(100, 16, seed=5)
    io.write_fvecs(str(tmp_path / "a.fvecs"), x)
    assert np.array_equal(io.read_fvecs(str(tmp_path / "a.fvecs")), x)
    ids = np.arange(30, dtype=np.int32).reshape(10, 3)
    io.write_ivecs(str(tmp_path / "a.ivecs"), ids)
    assert np.array_equal(io.read_ivecs(str(tmp_path / "a.ivecs")), ids)


def test_graph_csr_variable_degree(tmp_path):
    raw = np.array([2, 5, 6, 0, 3, 1, 2, 3], np.uint32)
    raw.tofile(str(tmp_path / "g.graph"))
    ptr, ids = io.read_graph_csr(str(tmp_path / "g.graph"))
    assert list(ptr) == [0, 2, 2, 5] and list(ids) == [5, 6, 1, 2, 3]


def test_generators_are_integer_valued_and_seeded():
    a = datasets.mixture_u8(500, 128, seed=0)
    b = datasets.mixture_u8(500, 128, seed=0)
    q = datasets.mixture_u8(50, 128, seed=0, queries=True)
    assert np.array_equal(a, b) and a.min() >= 0 and a.max() <= 255
    assert np.array_equal(a, np.rint(a)) and not np.array_equal(a[:50], q)
    u = datasets.mixture_unit(64, 960)
    assert u.min() >= 0 and u.max() <= 1
    assert np.allclose(u.reshape(64, 60, 16).sum(2), 1, atol=1e-5)


def test_code_files_roundtrip_and_shift(tmp_path):
    """The hashing initialiser's code files: 32-bit words up to 32 bits, 64-bit words above, the
    shift drops low bits, and a code longer than the length allowed is rejected."""
    import pytest
    rng = np.random.default_rng(0)
    for clen in (12, 32, 40, 64):
        c = rng.integers(0, 2 ** min(clen, 63), (3, 50), dtype=np.uint64)
        pre = str(tmp_path / ("c%d" % clen))
        io.write_codes(pre, c, clen)
        raw = np.fromfile(pre + "_2", np.int32)
        assert list(raw[:3]) == [1, clen, 50] and raw.size == 3 + 50 * (2 if clen > 32 else 1)
        back, bits = io.read_codes(pre, 3, clen)
        assert bits == clen and np.array_equal(back, c)
        back, bits = io.read_codes(pre, 3, clen, shift=3)
        assert bits == clen - 3 and np.array_equal(back, c >> np.uint64(3))
    pre = str(tmp_path / "bad")
    io.write_codes(pre, np.array([[1, 1 << 20]], np.uint64), 24)
    with pytest.raises(ValueError):
        io.read_codes(pre, 1, 16)  # the index parameter allows 16 bits


def test_sign_codes_seeded():
    x = datasets.mixture_u8(500, 16, seed=4)
    a = datasets.sign_codes(x, 3, 20, seed=7)
    b = datasets.sign_codes(x, 3, 20, seed=7)
    assert a.shape == (3, 500) and a.dtype == np.uint64 and np.array_equal(a, b)
    assert a.max() < 2 ** 20 and len(np.unique(a[0])) > 50
