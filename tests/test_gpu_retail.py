"""The benchmark's own workload against the reference and the oracle.

The plain-at-scale workload (retail graph: U = 1,000,000 users, I = 300,000
items, C = 2,000 categories, T = 20,000 tags, 20M U-I edges, 46.6M
adjacency entries) and its four chains I-T-I-C, C-I-U-I-C, T-I-C-I-T and
C-I-T-I-U-I-C run exactly as the benchmark runs them (uint32 counts widened
to uint64 on overflow, every bin and the tensor-core part where they apply):

* structure and nnz of every result: bit-identical to the reference's own
  rows (fixture made by efficient/resmcm.cpp itself, tests/golden);
* estimates within 1e-9 relative of the reference's one-thread c_, and the
  multiplication order equal to the reference's (both from the fixture);
* integer path counts: the result's order-free digest equals the counting
  oracle's on the same graph (exact uint64 counts).
"""
import numpy as np
import pytest

from helpers import adjacency_sha, load_fixture, make_graph, min_decision_gap, structure_sha

pytestmark = pytest.mark.gpu

EST_RTOL = 1e-9


@pytest.fixture(scope="module")
def retail(native, engine):
    fx = load_fixture("retail_full")
    g = make_graph(fx)
    assert adjacency_sha(g) == fx["adjacency_sha256"], "the generator no longer makes the fixture's graph"
    hg = native.HeteroGraph.from_synthetic(engine, g)
    yield fx, g, hg
    hg.close()


def test_retail_structure_and_nnz_match_reference(native, engine, retail):
    fx, _, hg = retail
    for rec in fx["paths"]:
        C, t, rc = engine.run_metapath(hg, rec["metapath"])
        assert rc == native.OK, rec["metapath"]
        assert C.nnz == rec["nnz"] == t["nnz"], rec["metapath"]
        rp, col, _ = C.download(values=False)
        C.free()
        assert rp.size - 1 == rec["rows"]
        assert structure_sha(rp, col) == rec["structure_sha256"], rec["metapath"]


def test_retail_estimates_and_order_match_reference(engine, retail):
    fx, _, hg = retail
    for rec in fx["paths"]:
        c = engine.estimate(hg.leaves(rec["metapath"]))
        ref = np.array(rec["c"])
        nz = ref != 0
        assert np.array_equal(c[~nz], ref[~nz]), rec["metapath"]
        rel = np.abs(c[nz] - ref[nz]) / np.abs(ref[nz])
        assert rel.max(initial=0.0) <= EST_RTOL, (rec["metapath"], rel.max())
        s, _, pairs = engine.order(c)
        if min_decision_gap(ref) >= EST_RTOL:
            assert s.tolist() == rec["split"] and pairs.tolist() == rec["pairs"], rec["metapath"]


def test_retail_path_counts_match_counting_oracle(engine, retail, oracle_mod):
    import os
    fx, g, hg = retail
    og = oracle_mod.OracleGraph.from_synthetic(g)
    for rec in fx["paths"]:
        C, _, _ = engine.run_metapath(hg, rec["metapath"])
        n_gpu, d_gpu = engine.digest(C)
        C.free()
        r = og.chain(rec["metapath"], oracle_mod.MODE_COUNT, threads=os.cpu_count() or 1, export=False,
                     digest=True)
        assert r.status == oracle_mod.ORC_OK, rec["metapath"]
        assert n_gpu == r.nnz == rec["nnz"], rec["metapath"]
        assert d_gpu == r.digest, rec["metapath"]
    og.close()
