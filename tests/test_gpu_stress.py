"""The memory-bound stress chain (twelve matrices over the X/Y/Z graph with
both-side Zipf(1.6) X-Y degrees, uint64 counts) at a size the counting oracle
finishes in seconds: results equal the oracle's, in uint64 and in AUTO mode,
and the RES order keeps every intermediate far below left-to-right."""
import numpy as np
import pytest

from resmcm_ari_gb300 import csr_digest, workloads

pytestmark = pytest.mark.gpu


def test_stress_chain_matches_the_counting_oracle(native, oracle_mod):
    g = workloads.stress_scaled(0.01)
    og = oracle_mod.OracleGraph.from_synthetic(g)
    r = og.chain(workloads.STRESS_CHAIN, mode=oracle_mod.MODE_COUNT, threads=8)
    want = csr_digest(r.rowptr, r.col, r.val)
    og.close()
    for vt in (native.VAL_U64, native.VAL_AUTO):
        eng = native.Engine(device=0, valtype=vt)
        hg = native.HeteroGraph.from_synthetic(eng, g)
        C, t, rc = eng.run_metapath(hg, workloads.STRESS_CHAIN)
        assert rc == native.OK
        assert eng.digest(C) == want
        C.free()
        hg.close()
        eng.close()


def test_stress_order_bounds_the_intermediates(native):
    g = workloads.stress_scaled(0.01)
    eng = native.Engine(device=0, valtype=native.VAL_U64)
    hg = native.HeteroGraph.from_synthetic(eng, g)
    leaves = hg.leaves(workloads.STRESS_CHAIN, native.VAL_U64)
    c = eng.estimate(leaves)
    split, _, _ = eng.order(c)
    L = c.shape[0]
    inter = []

    def walk(i, j):
        if i == j:
            return
        k = int(split[i, j])
        walk(i, k)
        walk(k + 1, j)
        inter.append(c[i, j])

    walk(0, L - 1)
    l2r = [c[0, j] for j in range(1, L)]
    assert max(inter) < max(l2r)
    hg.close()
    eng.close()
