"""Ablation orders on the host side of the C ABI (CPU only).

The dense-dimension DP is pinned by fixtures made by the reference's
efficient/naive.cpp itself (its DynamicOptimizer on each meta-path's type
dimensions), including its 32-bit int cost products: the full-size A-P-V-P-A
chain has dimension products above 2^31.
"""
import numpy as np
import pytest

from helpers import FIXTURES, load_fixture, make_graph


@pytest.mark.parametrize("name", FIXTURES)
def test_dense_order_matches_reference(native, name):
    fx = load_fixture(name)
    g = make_graph(fx)
    checked = 0
    for rec in fx["paths"]:
        if rec["len"] < 2:
            continue
        vts = native.MetaPath(rec["metapath"]).vertex_types
        dims = [g.type_sizes[t] if t < len(g.type_sizes) else 0 for t in vts]
        split, cost, pairs = native.order_dense(dims)
        assert split.tolist() == rec["dense_split"], rec["metapath"]
        assert np.array_equal(cost, np.array(rec["dense_m"])), rec["metapath"]
        assert pairs.tolist() == rec["dense_pairs"], rec["metapath"]
        checked += 1
    assert checked > 0


def test_l2r_order():
    import resmcm_ari_gb300 as rg
    rg.build()
    assert rg.order_l2r(2).tolist() == [[0, 1]]
    assert rg.order_l2r(5).tolist() == [[0, 1], [-1, 2], [-1, 3], [-1, 4]]
