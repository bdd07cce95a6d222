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
