"""GPU path (through the C ABI) against the reference fixtures and the oracle.

* structure and nnz of every result: bit-identical to the reference's rows
  (golden fixtures made by the reference itself);
* estimates: within 1e-9 relative of the reference's c_ (one-thread sums);
* the warp DP on the reference's own estimates: split table, costs and
  pair list bit-identical; the end-to-end order equals the reference's unless
  the reference itself sits on a near-tie (< 1e-9 relative);
* integer path counts: identical to the counting oracle;
* every parenthesisation of a chain gives the same CSR (exact integers).
"""
import itertools

import numpy as np
import pytest

from helpers import FIXTURES, load_fixture, make_graph, min_decision_gap, structure_sha

pytestmark = pytest.mark.gpu

EST_RTOL = 1e-9

_graphs = {}


def graph_for(native, engine, name):
    key = (name, id(engine))
    if key not in _graphs:
        fx = load_fixture(name)
        g = make_graph(fx)
        _graphs[key] = (fx, g, native.HeteroGraph.from_synthetic(engine, g))
    return _graphs[key]


@pytest.mark.parametrize("name", FIXTURES)
def test_structure_and_nnz_match_reference(native, engine, name):
    fx, _, hg = graph_for(native, engine, name)
    for rec in fx["paths"]:
        C, t, rc = engine.run_metapath(hg, rec["metapath"])
        assert rc == native.OK
        assert C.nnz == rec["nnz"] == t["nnz"], rec["metapath"]
        rp, col, _ = C.download(values=False)
        assert rp.size - 1 == rec["rows"]
        assert structure_sha(rp, col) == rec["structure_sha256"], rec["metapath"]
        if "rowptr" in rec:
            assert rp.tolist() == rec["rowptr"] and col.tolist() == rec["col"]
        C.free()


@pytest.mark.parametrize("name", FIXTURES)
def test_estimates_match_reference(native, engine, name):
    fx, _, hg = graph_for(native, engine, name)
    for rec in fx["paths"]:
        if rec["len"] < 2:
            continue
        c = engine.estimate(hg.leaves(rec["metapath"]))
        ref = np.array(rec["c"])
        nz = ref != 0
        assert np.array_equal(c[~nz], ref[~nz]), rec["metapath"]
        rel = np.abs(c[nz] - ref[nz]) / np.abs(ref[nz])
        assert rel.max(initial=0.0) <= EST_RTOL, (rec["metapath"], rel.max())


@pytest.mark.parametrize("name", FIXTURES)
def test_warp_dp_is_exact_on_reference_estimates(engine, name):
    fx = load_fixture(name)
    for rec in fx["paths"]:
        if rec["len"] < 2:
            continue
        s, m, pairs = engine.order(np.array(rec["c"]))
        assert s.tolist() == rec["split"], rec["metapath"]
        assert np.array_equal(m, np.array(rec["m"])), rec["metapath"]
        assert pairs.tolist() == rec["pairs"], rec["metapath"]


@pytest.mark.parametrize("name", FIXTURES)
def test_end_to_end_order_matches_reference(native, engine, name):
    fx, _, hg = graph_for(native, engine, name)
    for rec in fx["paths"]:
        if rec["len"] < 2:
            continue
        c = engine.estimate(hg.leaves(rec["metapath"]))
        _, _, pairs = engine.order(c)
        if pairs.tolist() != rec["pairs"]:
            assert min_decision_gap(rec["c"]) < EST_RTOL, rec["metapath"]


@pytest.mark.parametrize("name", FIXTURES)
def test_values_equal_counting_oracle(native, engine, oracle_mod, name):
    fx, g, hg = graph_for(native, engine, name)
    og = oracle_mod.OracleGraph.from_synthetic(g)
    for rec in fx["paths"]:
        ref = og.chain(rec["metapath"], oracle_mod.MODE_COUNT, threads=8)
        C, t, rc = engine.run_metapath(hg, rec["metapath"])
        rp, col, val = C.download()
        assert np.array_equal(rp, ref.rowptr), rec["metapath"]
        assert np.array_equal(col, ref.col), rec["metapath"]
        assert np.array_equal(val.astype(np.uint64), ref.val), rec["metapath"]
        C.free()


def all_orders(i, j):
    """Every parenthesisation of M_i..M_j as (tree result, pair list)."""
    if i == j:
        yield i, []
        return
    for k in range(i, j):
        for lres, lp in all_orders(i, k):
            for rres, rp in all_orders(k + 1, j):
                yield -1, lp + rp + [(lres, rres)]


@pytest.mark.parametrize("name,idx", [("dblp_small", 0), ("dblp_small", 5), ("hin4_small", 1), ("hin4_small", 4),
                                      ("tiny_dblp", 2)])
def test_every_parenthesisation_same_result(native, engine, name, idx):
    fx, _, hg = graph_for(native, engine, name)
    rec = fx["paths"][idx]
    leaves = hg.leaves(rec["metapath"])
    ref = None
    for _, pairs in all_orders(0, len(leaves) - 1):
        C, _, _ = engine.chain(leaves, pairs=np.array(pairs, np.int32))
        got = C.download()
        C.free()
        if ref is None:
            ref = got
            assert structure_sha(got[0], got[1]) == rec["structure_sha256"]
        else:
            for a, b in zip(ref, got):
                assert np.array_equal(a, b), (rec["metapath"], pairs)


@pytest.mark.parametrize("name", ["dblp_small", "hin4_small"])
def test_uint64_equals_uint32(native, engine, name):
    fx, _, hg = graph_for(native, engine, name)
    for rec in fx["paths"][:6]:
        C32, _, _ = engine.chain(hg.leaves(rec["metapath"], native.VAL_U32))
        C64, _, _ = engine.chain(hg.leaves(rec["metapath"], native.VAL_U64))
        a, b = C32.download(), C64.download()
        assert C64.valtype == native.VAL_U64
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
        assert np.array_equal(a[2].astype(np.uint64), b[2])
        C32.free()
        C64.free()


def test_run_twice_is_deterministic(native, engine):
    fx, _, hg = graph_for(native, engine, "config0_full")
    rec = fx["paths"][0]
    outs = []
    for _ in range(2):
        C, _, _ = engine.run_metapath(hg, rec["metapath"])
        outs.append(C.download())
        C.free()
    for a, b in zip(*outs):
        assert np.array_equal(a, b)
