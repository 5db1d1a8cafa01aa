"""Integer path counts of the oracle against scipy.sparse (independent check).

The reference is Boolean and cannot pin values; the counting oracle is pinned
here against scipy's int64 sparse products of the same leaf matrices, in the
chosen order and left to right (exact integer products are associative).
"""
import numpy as np
import pytest
import scipy.sparse as sp

from helpers import load_fixture, make_graph


def leaf_csr(og, vts, ets, i):
    rows, cols = og.dim(int(vts[i])), og.dim(int(vts[i + 1]))
    rp, col = og.leaf(int(vts[i]), int(vts[i + 1]), int(ets[i]))
    return sp.csr_matrix((np.ones(col.size, np.int64), col, rp), shape=(rows, cols))


@pytest.mark.parametrize("name", ["tiny_dblp", "dblp_small", "hin4_small"])
def test_counts_equal_scipy(oracle_mod, name):
    fx = load_fixture(name)
    og = oracle_mod.OracleGraph.from_synthetic(make_graph(fx))
    for rec in fx["paths"][:8]:
        if rec["nnz"] > 5_000_000:
            continue
        vts, ets = oracle_mod.parse_metapath(rec["metapath"])
        mats = [leaf_csr(og, vts, ets, i) for i in range(ets.size)]
        ref = mats[0]
        for M in mats[1:]:
            ref = ref @ M
        ref = ref.tocsr()
        ref.sum_duplicates()
        ref.sort_indices()
        r = og.chain(rec["metapath"], oracle_mod.MODE_COUNT, threads=2)
        assert np.array_equal(r.rowptr, ref.indptr), rec["metapath"]
        assert np.array_equal(r.col, ref.indices), rec["metapath"]
        assert np.array_equal(r.val.astype(np.int64), ref.data), rec["metapath"]


def test_repeated_neighbours_count_twice(oracle_mod):
    """A vertex listed twice with the same edge type is two paths (leaf rows keep repeats)."""
    # P0 -> A0 twice (edge type 0), A0 -> P0 twice (edge type 3)
    vtype = np.array([0, 1], np.int32)
    ptr = np.array([0, 2, 4], np.int64)
    nbr = np.array([1, 1, 0, 0], np.int32)
    et = np.array([0, 0, 3, 3], np.int32)
    og = oracle_mod.OracleGraph.from_arrays(vtype, ptr, nbr, et)
    r = og.chain("1-3-0-0-1", oracle_mod.MODE_COUNT)
    assert r.nnz == 1 and r.val.tolist() == [4]
    rb = og.chain("1-3-0-0-1", oracle_mod.MODE_BOOL)
    assert rb.nnz == 1
