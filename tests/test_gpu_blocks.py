"""Results delivered in blocks of rows (rmcm_run_metapath_blocks).

The final product of a chain is computed a block of rows at a time and each
block handed to the caller, so a result larger than the device memory left
under the budget never exists whole on the device:

* blocks of a fixed height put back together equal rmcm_run_metapath's
  result exactly, and their row-offset digests add up to its digest;
* under a budget too small for the whole result, the plain call fails and
  the blocked one (block height from the RES estimate and the free budget)
  matches the reference's nnz and the counting oracle's exact path counts;
* in AUTO mode, rows whose counts fit uint32 come back as uint32 and, after
  the first block that overflows, the rest as uint64, every value exact.
"""
import numpy as np
import pytest

from helpers import load_fixture, make_graph
from resmcm_ari_gb300 import synth

pytestmark = pytest.mark.gpu


def _collect(engine, hg, mp, rows_per_block=0):
    blocks = []

    def on_block(row0, blk):
        rp, col, val = blk.download()
        n, d = engine.digest_rows(blk, row0)
        blocks.append((row0, rp, col, val.astype(np.uint64), blk.valtype, n, d))

    t, rc = engine.run_metapath_blocks(hg, mp, on_block, rows_per_block)
    return blocks, t, rc


def _concat(blocks, rows):
    rp = [np.zeros(1, np.int64)]
    cols, vals = [], []
    base = 0
    expect = 0
    for row0, brp, col, val, _, _, _ in blocks:
        assert row0 == expect
        rp.append(brp[1:] + base)
        base += int(brp[-1])
        expect = row0 + brp.size - 1
        cols.append(col)
        vals.append(val)
    assert expect == rows
    return np.concatenate(rp), np.concatenate(cols), np.concatenate(vals)


def test_fixed_blocks_equal_the_whole_result(native, engine):
    fx = load_fixture("dblp_small")
    hg = native.HeteroGraph.from_synthetic(engine, make_graph(fx))
    for rec in fx["paths"]:
        C, _, rc = engine.run_metapath(hg, rec["metapath"])
        rp, col, val = C.download()
        want_digest = engine.digest(C)
        C.free()
        for rb in (37, 1000):
            blocks, t, rc2 = _collect(engine, hg, rec["metapath"], rb)
            assert rc2 == rc and t["nnz"] == rec["nnz"]
            brp, bcol, bval = _concat(blocks, rp.size - 1)
            assert np.array_equal(brp, rp) and np.array_equal(bcol, col)
            assert np.array_equal(bval, val.astype(np.uint64)), rec["metapath"]
            assert sum(b[5] for b in blocks) == want_digest[0]
            assert sum(b[6] for b in blocks) % (1 << 64) == want_digest[1]


def test_budget_sized_blocks_fit_where_the_whole_result_does_not(native, oracle_mod):
    fx = load_fixture("config0_full")
    g = make_graph(fx)
    rec = fx["paths"][0]
    budget = 512 << 20          # the result alone needs ~0.9 GB
    eng = native.Engine(device=0, mem_budget_bytes=budget)
    hg = native.HeteroGraph.from_synthetic(eng, g)
    with pytest.raises(native.RmcmError) as e:
        eng.run_metapath(hg, rec["metapath"])
    assert e.value.status == native.ENOMEM
    eng.mem_peak(reset=True)
    state = {"n": 0, "d": 0, "blocks": 0}

    def on_block(row0, blk):
        n, d = eng.digest_rows(blk, row0)
        state["n"] += n
        state["d"] = (state["d"] + d) % (1 << 64)
        state["blocks"] += 1

    t, rc = eng.run_metapath_blocks(hg, rec["metapath"], on_block)
    assert rc == native.OK and state["blocks"] > 1
    assert state["n"] == t["nnz"] == rec["nnz"]
    assert eng.mem_peak() <= budget
    ref = oracle_mod.OracleGraph.from_synthetic(g).chain(rec["metapath"], oracle_mod.MODE_COUNT, threads=8,
                                                         export=False, digest=True)
    assert ref.digest == state["d"]
    hg.close()
    eng.close()


def test_auto_blocks_widen_where_counts_overflow(native, oracle_mod):
    # X3 links to all 3,000 Y (and every Y back to it); X0..X2 to two Y
    # each: along X-Y-X-Y-X-Y-X only X3's row passes 2^32 (3000^3 paths)
    ny = 3000
    src = np.concatenate([np.full(ny, 3, np.int64), np.repeat(np.arange(3, dtype=np.int64), 2)])
    dst = np.concatenate([np.arange(ny, dtype=np.int64), np.arange(6, dtype=np.int64)])
    g = synth.SyntheticHIN("hub", [4, ny], [synth.Relation(0, 1, 0, 1, src, dst)])
    mp = "0-0-1-1-0-0-1-1-0-0-1-1-0"
    eng = native.Engine(device=0, valtype=native.VAL_AUTO)
    hg = native.HeteroGraph.from_synthetic(eng, g)
    blocks, t, rc = _collect(eng, hg, mp, 1)
    assert rc == native.OK
    assert [b[4] for b in blocks] == [native.VAL_U32] * 3 + [native.VAL_U64]
    rp, col, val = _concat(blocks, 4)
    ref = oracle_mod.OracleGraph.from_synthetic(g).chain(mp, oracle_mod.MODE_COUNT, threads=2)
    assert np.array_equal(rp, ref.rowptr) and np.array_equal(col, ref.col)
    assert np.array_equal(val, ref.val) and int(val.max()) > (1 << 32)
    hg.close()
    eng.close()
