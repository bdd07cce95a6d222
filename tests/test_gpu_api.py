"""The public API and file formats on the GPU: reference-shaped CLI, save/load round trips,
graph rows and error codes."""
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, load_golden
from efanna_gb300 import datasets, io

pytestmark = pytest.mark.gpu


def _cli():
    from efanna_gb300 import build
    return build.build_cli()


def test_cli_pipeline_matches_api(efg, tmp_path):
    x = datasets.mixture_u8(3000, 32, seed=2)
    q = datasets.mixture_u8(100, 32, seed=2, queries=True)
    base, qf = str(tmp_path / "b.fvecs"), str(tmp_path / "q.fvecs")
    io.write_fvecs(base, x)
    io.write_fvecs(qf, q)
    cli = _cli()
    g, t, r = str(tmp_path / "g.graph"), str(tmp_path / "t.trees"), str(tmp_path / "r.ivecs")
    run = lambda *a: subprocess.run([cli] + list(a), capture_output=True, text=True)
    p = run("efanna_index_buildall", base, g, t, "8", "4", "8", "30", "25", "10", "10")
    assert p.returncode == 0, p.stdout + p.stderr
    p = run("efanna_search", base, t, g, qf, r, "8", "4", "300", "60", "10")
    assert p.returncode == 0, p.stdout + p.stderr
    idx = efg.Index(x, efg.IndexParams(trees=8, merge_level=4, epochs=8, check=25, L=30, K=10, S=10))
    idx.build_index()
    ref_graph = np.fromfile(g, np.uint32).reshape(3000, 11)
    assert np.array_equal(ref_graph[:, 1:], idx.graph())
    idx.set_search_params(4, 300, 60, 8)
    assert np.array_equal(io.read_ivecs(r), idx.knn_search(10, q))
    io.write_ivecs(str(tmp_path / "gt.ivecs"), io.read_ivecs(r))
    p = run("evaluate", r, str(tmp_path / "gt.ivecs"), "10")
    assert "10NN accuracy: 1" in p.stdout
    p = run("efanna_index_buildtrees", base, str(tmp_path / "t16.trees"), "16")
    assert p.returncode == 0 and os.path.getsize(str(tmp_path / "t16.trees")) > 16 * 3000 * 4


def test_file_roundtrips(efg, tmp_path):
    g = load_golden("mid_d128")
    x = g["base"].astype(np.float32)
    q = g["queries"].astype(np.float32)
    idx = efg.Index(x, efg.IndexParams(trees=8, merge_level=5, epochs=6))
    idx.build_index()
    idx.set_search_params(4, 600, 100, 8)
    res = idx.knn_search(10, q)
    for name in ("graph", "trees", "index"):
        getattr(idx, "save_" + name)(str(tmp_path / name))
    idx.save_results(str(tmp_path / "res.ivecs"))
    assert np.array_equal(io.read_ivecs(str(tmp_path / "res.ivecs")), res)
    # graph file is the reference's layout: per row u32 k then k ids
    raw = np.fromfile(str(tmp_path / "graph"), np.uint32).reshape(len(x), 11)
    assert np.all(raw[:, 0] == 10) and np.array_equal(raw[:, 1:], idx.graph())
    assert idx.graph_size() == len(x) and idx.graph_row(7) == list(raw[7, 1:])
    assert idx.graph_row(len(x) + 5) == []
    # reload into fresh indexes
    b = efg.Index(x, efg.IndexParams(trees=8))
    b.load_trees(str(tmp_path / "trees"))
    b.load_graph(str(tmp_path / "graph"))
    b.set_search_params(4, 600, 100, 8)
    assert np.array_equal(b.knn_search(10, q), res)
    c = efg.Index(x, efg.IndexParams(trees=8))
    c.load_index(str(tmp_path / "index"))
    c.set_search_params(4, 600, 100, 8)
    assert np.array_equal(c.knn_search(10, q), res)
    # trees saved after a load are byte-identical
    b.save_trees(str(tmp_path / "trees2"))
    assert open(tmp_path / "trees", "rb").read() == open(tmp_path / "trees2", "rb").read()


def test_loaded_reference_files_roundtrip_bytes(efg, tmp_path):
    g = load_golden("small_d32")
    x = g["base"].astype(np.float32)
    idx = efg.Index(x, efg.IndexParams(trees=8))
    idx.load_graph(os.path.join(GOLDEN, "small_d32.graph"))
    idx.save_graph(str(tmp_path / "g"))
    assert open(tmp_path / "g", "rb").read() == open(os.path.join(GOLDEN, "small_d32.graph"), "rb").read()


def test_open_and_format_errors(efg, tmp_path):
    x = datasets.mixture_u8(500, 16, seed=1)
    idx = efg.Index(x, efg.IndexParams(trees=2, merge_level=2))
    for fn in (idx.load_graph, idx.load_trees, idx.load_index):
        with pytest.raises(efg.EfannaError) as e:
            fn(str(tmp_path / "missing"))
        assert e.value.code == efg.EFG_ERR_OPEN
    (tmp_path / "trunc").write_bytes(b"\x0a\x00\x00\x00\x01\x00")
    with pytest.raises(efg.EfannaError) as e:
        idx.load_trees(str(tmp_path / "trunc"))
    assert e.value.code == efg.EFG_ERR_FORMAT
    bad = np.array([[2, 1, 999999]] * 500, np.uint32)
    bad.tofile(str(tmp_path / "badgraph"))
    with pytest.raises(efg.EfannaError) as e:
        idx.load_graph(str(tmp_path / "badgraph"))
    assert e.value.code == efg.EFG_ERR_FORMAT
    with pytest.raises(efg.EfannaError) as e:
        idx.save_graph(str(tmp_path / "nograph"))
    assert e.value.code == efg.EFG_ERR_STATE and os.path.getsize(str(tmp_path / "nograph")) == 0


def test_device_resident_index_and_stats(efg):
    torch = pytest.importorskip("torch")
    x = datasets.mixture_u8(4000, 64, seed=9)
    X = torch.from_numpy(x).cuda()
    a = efg.Index.from_device(X.data_ptr(), 4000, 64, 64, efg.IndexParams(trees=4, merge_level=4, epochs=5))
    b = efg.Index(x, efg.IndexParams(trees=4, merge_level=4, epochs=5))
    a.build_index()
    b.build_index()
    assert np.array_equal(a.graph(), b.graph())
    s = a.build_stats()
    assert s.join_pairs > 0 and s.merge_distances > 0 and s.total_ms > 0 and s.trees_ms > 0


def test_graph_csc_is_the_transpose_of_the_graph(efg):
    """getGraphMat (matlab/findex.cc:106-150): column j lists, ascending, the nodes whose rows hold j."""
    x = datasets.mixture_u8(3000, 32, seed=4)
    idx = efg.Index(x, efg.IndexParams(trees=4, merge_level=4, epochs=4))
    idx.build_index()
    g = idx.graph()
    col_ptr, row_ids = idx.graph_csc()
    assert col_ptr[-1] == g.size
    src = np.repeat(np.arange(g.shape[0], dtype=np.uint32), g.shape[1])
    order = np.lexsort((src, g.ravel()))  # by column, then by row
    assert np.array_equal(row_ids, src[order])
    assert np.array_equal(col_ptr[1:], np.cumsum(np.bincount(g.ravel(), minlength=g.shape[0])))
