"""The graph's compressed-column export (the MATLAB front end's getGraphMat, matlab/findex.cc:106-150):
the host transpose in the C ABI against a restatement of the reference's loop, with no GPU."""
import numpy as np
import pytest


def _reference_csc(row_ptr, ids, n):
    """findex.cc:106-150: for every row i in order, append i to the column of each id in row i; then
    the columns in order, empty ones included."""
    cols = {}
    for i in range(n):
        for x in ids[row_ptr[i]:row_ptr[i + 1]]:
            cols.setdefault(int(x), []).append(i)
    jc, ir = [0], []
    for j in range(n):
        ir.extend(cols.get(j, []))
        jc.append(len(ir))
    return np.array(jc, np.uint64), np.array(ir, np.uint32)


@pytest.mark.parametrize("n,maxdeg,seed", [(1, 3, 0), (50, 0, 1), (500, 12, 2), (3000, 40, 3)])
def test_csr_transpose_matches_reference_loop(efg, n, maxdeg, seed):
    rng = np.random.default_rng(seed)
    deg = rng.integers(0, maxdeg + 1, n)
    row_ptr = np.concatenate([[0], np.cumsum(deg)]).astype(np.uint64)
    ids = rng.integers(0, n, int(row_ptr[-1])).astype(np.uint32)  # repeats and self ids included
    jc, ir = efg.csr_transpose(row_ptr, ids, n)
    rjc, rir = _reference_csc(row_ptr, ids, n)
    assert np.array_equal(jc, rjc) and np.array_equal(ir, rir)


def test_csr_transpose_rejects_ids_out_of_range(efg):
    with pytest.raises(efg.EfannaError):
        efg.csr_transpose(np.array([0, 2, 3], np.uint64), np.array([0, 2, 1], np.uint32), 2)
    with pytest.raises(efg.EfannaError):
        efg.csr_transpose(np.array([0, 2, 1], np.uint64), np.array([0, 1], np.uint32), 2)
