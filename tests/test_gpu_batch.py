"""Batches (rmcm_batch_*): many meta-paths recorded once and replayed as one
CUDA graph over concurrent lanes.  Every path's result must equal, entry for
entry, what rmcm_run_metapath gives alone and what the counting oracle gives:
compared through the order-free digest (nnz + 64-bit entry hash)."""
import numpy as np
import pytest

from helpers import load_fixture, make_graph
from resmcm_ari_gb300 import csr_digest, synth

pytestmark = pytest.mark.gpu


def _plain_digests(native, eng, hg, paths):
    out = []
    for mp in paths:
        C, _, rc = eng.run_metapath(hg, mp)
        assert rc == native.OK, mp
        d = eng.digest(C)
        rp, col, val = C.download()
        assert d == csr_digest(rp, col, val), mp       # device digest == host definition
        C.free()
        out.append(d)
    return out


@pytest.mark.parametrize("lanes", [1, 4])
def test_batch_equals_plain_and_oracle(native, oracle_mod, lanes):
    fx = load_fixture("hin4_small")
    g = make_graph(fx)
    paths = [r["metapath"] for r in fx["paths"]]
    eng = native.Engine(device=0)
    hg = native.HeteroGraph.from_synthetic(eng, g)
    plain = _plain_digests(native, eng, hg, paths)
    og = oracle_mod.OracleGraph.from_synthetic(g)
    for mp, d in zip(paths, plain):
        r = og.chain(mp, mode=oracle_mod.MODE_COUNT, threads=4)
        assert csr_digest(r.rowptr, r.col, r.val) == d, mp
    og.close()
    b = eng.batch(hg, paths, lanes=lanes)
    info = b.info()
    assert info["count"] == len(paths) and info["lanes"] == min(lanes, len(paths))
    assert info["launches_per_run"] > 0
    for _ in range(3):                                   # the graph replays identically
        nnz, dig, sec = b.run()
        assert sec > 0
        assert [(int(n), int(x)) for n, x in zip(nnz, dig)] == plain
    b.free()
    hg.close()
    eng.close()


def test_batch_with_uint64_escalation_and_single_matrix_paths(native):
    """K(64,64) paths: the long ones overflow uint32 and escalate mid-chain
    in the record pass; the replay repeats the escalated plan."""
    n = 64
    src = np.repeat(np.arange(n), n)
    dst = np.tile(np.arange(n), n)
    g = synth.SyntheticHIN("k64", [n, n], [synth.Relation(0, 1, 0, 1, src, dst)])
    paths = ["0-0-1", "0-0-1-1-0", "0-0-1-1-0-0-1-1-0-0-1-1-0-0-1-1-0", "1-1-0-0-1-1-0-0-1-1-0"]
    eng = native.Engine(device=0, valtype=native.VAL_AUTO)
    hg = native.HeteroGraph.from_synthetic(eng, g)
    plain = _plain_digests(native, eng, hg, paths)
    b = eng.batch(hg, paths, lanes=2)
    for _ in range(2):
        nnz, dig, _ = b.run()
        assert [(int(a), int(x)) for a, x in zip(nnz, dig)] == plain
    # the graph's leaves stay while a batch replays them
    with pytest.raises(Exception):
        hg.close()
    b.free()
    hg.close()
    eng.close()


def test_batch_on_random_walks_of_a_five_type_graph(native):
    from resmcm_ari_gb300 import workloads
    g = workloads.batch_graph(seed=2, scale=1 / 400)
    paths = workloads.batch_walks(5, g, 48, lengths=(2, 6))
    eng = native.Engine(device=0)
    hg = native.HeteroGraph.from_synthetic(eng, g)
    plain = _plain_digests(native, eng, hg, paths)
    b = eng.batch(hg, paths, lanes=8)
    nnz, dig, _ = b.run()
    assert [(int(a), int(x)) for a, x in zip(nnz, dig)] == plain
    b.free()
    hg.close()
    eng.close()


def _fused_equals_plain(native, eng, hg, paths, reps=3):
    plain = _plain_digests(native, eng, hg, paths)
    b = eng.batch(hg, paths, fused=True)
    info = b.info()
    assert info["count"] == len(paths) and info["lanes"] == 1 and info["launches_per_run"] > 0
    for _ in range(reps):                                # the graph replays identically
        nnz, dig, sec = b.run()
        assert sec > 0
        assert [(int(n), int(x)) for n, x in zip(nnz, dig)] == plain
    b.free()
    return info


def test_fused_batch_equals_plain_and_oracle(native, oracle_mod):
    """Estimator levels, DP and one block-diagonal SpGEMM per wave shared by
    every chain: every result equals rmcm_run_metapath's and the counting
    oracle's, in far fewer launches than one chain at a time."""
    fx = load_fixture("hin4_small")
    g = make_graph(fx)
    paths = [r["metapath"] for r in fx["paths"]]
    eng = native.Engine(device=0)
    hg = native.HeteroGraph.from_synthetic(eng, g)
    og = oracle_mod.OracleGraph.from_synthetic(g)
    for mp in paths:
        r = og.chain(mp, mode=oracle_mod.MODE_COUNT, threads=4)
        C, _, _ = eng.run_metapath(hg, mp)
        assert csr_digest(r.rowptr, r.col, r.val) == eng.digest(C), mp
        C.free()
    og.close()
    info = _fused_equals_plain(native, eng, hg, paths)
    per_chain = eng.batch(hg, paths, lanes=1)
    assert info["launches_per_run"] * 3 < per_chain.info()["launches_per_run"]
    per_chain.free()
    hg.close()
    eng.close()


def test_fused_batch_with_uint64_escalation_and_single_matrix_paths(native):
    """K(64,64): long paths overflow uint32; the wave that overflows widens
    the whole batch to uint64 in the record, and the replay repeats it."""
    n = 64
    src = np.repeat(np.arange(n), n)
    dst = np.tile(np.arange(n), n)
    g = synth.SyntheticHIN("k64", [n, n], [synth.Relation(0, 1, 0, 1, src, dst)])
    paths = ["0-0-1", "0-0-1-1-0", "0-0-1-1-0-0-1-1-0-0-1-1-0-0-1-1-0", "1-1-0-0-1-1-0-0-1-1-0", "1-1-0"]
    eng = native.Engine(device=0, valtype=native.VAL_AUTO)
    hg = native.HeteroGraph.from_synthetic(eng, g)
    _fused_equals_plain(native, eng, hg, paths, reps=2)
    hg.close()
    eng.close()


@pytest.mark.parametrize("count,lengths", [(48, (2, 6)), (160, (2, 10))])
def test_fused_batch_on_random_walks_of_a_five_type_graph(native, count, lengths):
    from resmcm_ari_gb300 import workloads
    g = workloads.batch_graph(seed=2, scale=1 / 400)
    paths = workloads.batch_walks(5, g, count, lengths=lengths)
    eng = native.Engine(device=0)
    hg = native.HeteroGraph.from_synthetic(eng, g)
    _fused_equals_plain(native, eng, hg, paths, reps=2)
    hg.close()
    eng.close()


def test_bad_batch_arguments(native, engine):
    g = synth.tiny_dblp()
    hg = native.HeteroGraph.from_synthetic(engine, g)
    with pytest.raises(native.RmcmError):
        engine.batch(hg, ["0-0-1", "not-a-path"])
    engine.set_order_mode(native.ORDER_L2R)
    with pytest.raises(native.RmcmError):
        engine.batch(hg, ["0-0-1"])
    engine.set_order_mode(native.ORDER_RES)
    hg.close()


@pytest.mark.parametrize("tpr", [1, 2, 4, 8, 16, 32, 128])
def test_every_threads_per_row_gives_the_same_products(native, tpr):
    """Short rows through the micro bin (1..16 lanes), a warp, or a CTA."""
    fx = load_fixture("hin4_small")
    g = make_graph(fx)
    paths = [r["metapath"] for r in fx["paths"]]
    eng = native.Engine(device=0)
    hg = native.HeteroGraph.from_synthetic(eng, g)
    ref = _plain_digests(native, eng, hg, paths)
    eng.set_tuning(threads_per_row=tpr)
    assert _plain_digests(native, eng, hg, paths) == ref
    hg.close()
    eng.close()


@pytest.mark.parametrize("hash_max,load", [(32, 0.5), (128, 0.7), (512, 0.7), (8192, 0.5), (8192, 0.75)])
def test_bin_thresholds_and_load_factors_give_the_same_products(native, hash_max, load):
    rng = np.random.default_rng(hash_max)
    import scipy.sparse as sp
    A = sp.random(300, 4000, density=0.01, random_state=rng, format="csr", dtype=np.float64)
    B = sp.random(4000, 9000, density=0.004, random_state=rng, format="csr", dtype=np.float64)
    A.data[:] = rng.integers(1, 4, A.nnz)
    B.data[:] = rng.integers(1, 4, B.nnz)
    want = (A @ B).tocsr()
    want.sort_indices()
    eng = native.Engine(device=0)
    eng.set_tuning(hash_max_flops=hash_max, hash_load=load, threads_per_row=4)
    dA = eng.upload(A.indptr, A.indices, cols=A.shape[1], val=A.data.astype(np.uint64))
    dB = eng.upload(B.indptr, B.indices, cols=B.shape[1], val=B.data.astype(np.uint64))
    C = eng.spgemm(dA, dB)
    rp, col, val = C.download()
    assert np.array_equal(rp, want.indptr) and np.array_equal(col, want.indices)
    assert np.array_equal(val, want.data.astype(np.uint64))
    eng.close()


def test_autotuner_keeps_results_and_picks_a_measured_best(native):
    from resmcm_ari_gb300 import autotune, workloads
    g = workloads.batch_graph(seed=2, scale=1 / 400)
    paths = workloads.batch_walks(7, g, 32, lengths=(2, 6))
    eng = native.Engine(device=0)
    hg = native.HeteroGraph.from_synthetic(eng, g)
    res = autotune.tune(eng, hg, paths, lanes=4, reps=2, mode="coordinate")
    assert len(res["table"]) >= 8
    assert res["best_s"] == min(t for _, t, _ in res["table"])
    assert eng.get_tuning()["threads_per_row"] == res["best"]["threads_per_row"]
    hg.close()
    eng.close()


def test_bad_tuning_is_rejected(native, engine):
    for kw in ({"threads_per_row": 3}, {"hash_max_flops": 8}, {"hash_load": 0.9}, {"dense_ratio": 0},
               {"warp_max_flops": -1}, {"warp_max_flops": 70000}):
        with pytest.raises(native.RmcmError):
            engine.set_tuning(**kw)
    assert engine.get_tuning() == {"threads_per_row": 4, "hash_max_flops": 4096, "dense_ratio": 16,
                                   "warp_max_flops": 2048, "hash_load": 0.5, "gemm_inv_density": 512,
                                   "gemm_min_mflops": 512}


def test_fused_batch_at_the_configured_sizes_matches_the_oracle(native, oracle_mod):
    """The batched workload at its configured sizes (five types of 10k-500k
    vertices, 5-40 edges per row): the first 24 seeded walks whose RES
    prediction stays within 1 GB, as one fused batch, against the counting
    oracle's exact path counts on the same graph."""
    import os
    from resmcm_ari_gb300 import serve, workloads
    g = workloads.batch_graph(seed=2, scale=1.0)
    eng = native.Engine(device=0)
    hg = native.HeteroGraph.from_synthetic(eng, g)
    paths = []
    for mp in synth.random_metapaths(3, g, 256, (2, 10)):
        leaves = hg.leaves(mp)
        c = eng.estimate(leaves)
        split, _, _ = eng.order(c)
        dims = [m.shape[0] for m in leaves] + [leaves[-1].shape[1]]
        if serve.predicted_bytes(c, split, dims) <= 1e9:
            paths.append(mp)
        if len(paths) == 24:
            break
    assert len(paths) == 24
    b = eng.batch(hg, paths, fused=True)
    nnz, dig, _ = b.run()
    b.free()
    og = oracle_mod.OracleGraph.from_synthetic(g)
    for mp, n, d in zip(paths, nnz, dig):
        r = og.chain(mp, oracle_mod.MODE_COUNT, threads=os.cpu_count() or 1, export=False, digest=True)
        assert r.status == oracle_mod.ORC_OK and r.nnz == int(n) and r.digest == int(d), mp
    og.close()
    hg.close()
    eng.close()
