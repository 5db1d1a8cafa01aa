"""The CPU oracle against the reference's own outputs (golden fixtures).

These run on CPU only.  They pin the oracle: generator determinism, the text
loader, the estimator's FP64 sums (bit-identical to the reference at one
thread), the DP and order extraction, and the Boolean and counting products'
structure.
"""
import os
import tempfile

import numpy as np
import pytest

from helpers import FIXTURES, adjacency_sha, load_fixture, make_graph, structure_sha

SMALL = ["tiny_dblp", "dblp_small", "hin4_small"]


@pytest.mark.parametrize("name", FIXTURES)
def test_generator_is_the_fixture_graph(name):
    fx = load_fixture(name)
    g = make_graph(fx)
    assert g.n == fx["n"] and g.m == fx["m"]
    assert adjacency_sha(g) == fx["adjacency_sha256"]


@pytest.mark.parametrize("name", SMALL)
def test_text_loader_roundtrip(oracle_mod, name):
    fx = load_fixture(name)
    g = make_graph(fx)
    with tempfile.TemporaryDirectory() as d:
        files = g.write_text(d)
        og = oracle_mod.OracleGraph.from_text(files["graph"], files["vertex"], files["edge"])
    vt, ptr, nbr, et = og.export()
    p2, n2, e2 = g.adjacency()
    assert np.array_equal(vt, g.vertex_types())
    assert np.array_equal(ptr, p2) and np.array_equal(nbr, n2) and np.array_equal(et, e2)


@pytest.mark.parametrize("name", FIXTURES)
def test_estimates_bit_identical_at_one_thread(oracle_mod, name):
    fx = load_fixture(name)
    og = oracle_mod.OracleGraph.from_synthetic(make_graph(fx))
    for rec in fx["paths"]:
        if rec["len"] < 2:
            continue
        c = og.estimate(rec["metapath"], threads=1)
        assert np.array_equal(c, np.array(rec["c"])), rec["metapath"]


@pytest.mark.parametrize("name", FIXTURES)
def test_dp_and_order_match_reference(oracle_mod, name):
    fx = load_fixture(name)
    for rec in fx["paths"]:
        if rec["len"] < 2:
            continue
        m, s, pairs = oracle_mod.dp(np.array(rec["c"]))
        assert np.array_equal(s, np.array(rec["split"])), rec["metapath"]
        assert pairs.tolist() == rec["pairs"], rec["metapath"]
        assert np.array_equal(m, np.array(rec["m"])), rec["metapath"]


@pytest.mark.parametrize("name", FIXTURES)
@pytest.mark.parametrize("mode", ["bool", "count"])
def test_chain_structure_matches_reference(oracle_mod, name, mode):
    fx = load_fixture(name)
    og = oracle_mod.OracleGraph.from_synthetic(make_graph(fx))
    md = oracle_mod.MODE_BOOL if mode == "bool" else oracle_mod.MODE_COUNT
    for rec in fx["paths"]:
        r = og.chain(rec["metapath"], md, threads=4)
        assert r.nnz == rec["nnz"], rec["metapath"]
        assert structure_sha(r.rowptr, r.col) == rec["structure_sha256"], rec["metapath"]
        if "rowptr" in rec:
            assert r.rowptr.tolist() == rec["rowptr"] and r.col.tolist() == rec["col"]


def test_tiny_known_answers(oracle_mod):
    """Hand-checkable counts on the 8-vertex P/A/V graph."""
    fx = load_fixture("tiny_dblp")
    og = oracle_mod.OracleGraph.from_synthetic(make_graph(fx))
    # A-P-A co-authorship: author 0 wrote papers 0 and 2, author 1 papers 0 and 1,
    # author 2 papers 2 and 3.
    r = og.chain("1-3-0-0-1", oracle_mod.MODE_COUNT)
    dense = np.zeros((3, 3), np.uint64)
    for u in range(3):
        for q in range(r.rowptr[u], r.rowptr[u + 1]):
            dense[u, r.col[q]] = r.val[q]
    assert dense.tolist() == [[2, 1, 1], [1, 2, 0], [1, 0, 2]]
    # A-P-V-P-A: every pair of authors shares the single venue: 2 papers x 2 papers
    r = og.chain("1-3-0-1-2-4-0-0-1", oracle_mod.MODE_COUNT)
    assert r.nnz == 9 and set(r.val.tolist()) == {4}
