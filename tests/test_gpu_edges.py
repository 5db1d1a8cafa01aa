"""Edge cases of the GPU path: empty and ragged inputs, repeated neighbours,
chains of one matrix, overflow detection (uint32 and uint64), the automatic
uint64 re-run, bad arguments and the device memory budget."""
import os
import subprocess
import tempfile

import numpy as np
import pytest
import scipy.sparse as sp

from resmcm_ari_gb300 import synth

pytestmark = pytest.mark.gpu


def csr(dense):
    dense = np.asarray(dense)
    rp = [0]
    col, val = [], []
    for row in dense:
        nz = np.nonzero(row)[0]
        col += nz.tolist()
        val += row[nz].tolist()
        rp.append(len(col))
    return np.array(rp, np.int64), np.array(col, np.int32), np.array(val, np.uint64)


def test_repeated_neighbours_count_as_separate_paths(native, engine):
    vtype = np.array([0, 1], np.int32)
    hg = native.HeteroGraph.from_adjacency(engine, vtype, np.array([0, 2, 4]), np.array([1, 1, 0, 0]),
                                           np.array([0, 0, 3, 3]))
    C, t, _ = engine.run_metapath(hg, "1-3-0-0-1")
    rp, col, val = C.download()
    assert rp.tolist() == [0, 1] and col.tolist() == [0] and val.tolist() == [4]


def test_empty_result_and_empty_rows(native, engine):
    g = synth.tiny_dblp()
    hg = native.HeteroGraph.from_synthetic(engine, g)
    # edge type 9 does not exist: the leaf is empty, so is the product
    C, t, _ = engine.run_metapath(hg, "1-3-0-9-2-4-0")
    assert C.nnz == 0 and t["nnz"] == 0
    rp, col, _ = C.download()
    assert rp.tolist() == [0, 0, 0, 0]


def test_chain_of_one_matrix_is_the_leaf(native, engine):
    g = synth.tiny_dblp()
    hg = native.HeteroGraph.from_synthetic(engine, g)
    C, t, _ = engine.run_metapath(hg, "0-1-2")
    rp, col, val = C.download()
    assert rp.tolist() == [0, 1, 2, 3, 4] and col.tolist() == [0, 0, 0, 0] and val.tolist() == [1, 1, 1, 1]
    assert t["total_s"] == 0.0


def test_empty_matrices(native, engine):
    A = engine.upload(np.zeros(1, np.int64), np.zeros(0, np.int32), cols=5)
    B = engine.upload(np.zeros(6, np.int64), np.zeros(0, np.int32), cols=3)
    C = engine.spgemm(A, B)
    assert C.shape == (0, 3) and C.nnz == 0


def _check_product(native, engine, A, B, vt):
    A = A.tocsr(); B = B.tocsr()
    A.sort_indices(); B.sort_indices()
    ref = (A @ B).tocsr()
    ref.sum_duplicates(); ref.sort_indices()
    Am = engine.upload(A.indptr, A.indices, cols=A.shape[1], val=A.data.astype(np.uint64), valtype=vt)
    Bm = engine.upload(B.indptr, B.indices, cols=B.shape[1], val=B.data.astype(np.uint64), valtype=vt)
    Cm = engine.spgemm(Am, Bm)
    rp, col, val = Cm.download()
    assert np.array_equal(rp, ref.indptr) and np.array_equal(col, ref.indices)
    assert np.array_equal(val.astype(np.uint64), ref.data.astype(np.uint64))


def _random_csr(rng, m, n, row_nnz, vmax=3):
    rows, cols = [], []
    for r in range(m):
        k = int(row_nnz[r])
        rows += [r] * k
        cols += rng.choice(n, k, replace=False).tolist()
    data = rng.integers(1, vmax + 1, len(rows))
    return sp.csr_matrix((data.astype(np.int64), (rows, cols)), shape=(m, n))


def test_products_in_every_bin_match_scipy(native, engine):
    """Rows spanning the tiny, hash and dense bins, with empty rows."""
    rng = np.random.default_rng(5)
    m, k, n = 300, 400, 20000
    a_nnz = np.linspace(0, 120, m).astype(int)
    a_nnz[::7] = 0
    A = _random_csr(rng, m, k, a_nnz)
    B = _random_csr(rng, k, n, rng.integers(0, 400, k))
    for vt in (native.VAL_U32, native.VAL_U64):
        _check_product(native, engine, A, B, vt)


def test_hash_bins_with_wide_columns(native, engine):
    rng = np.random.default_rng(6)
    m, k, n = 500, 3000, 5_000_000
    A = _random_csr(rng, m, k, rng.integers(1, 60, m))
    B = _random_csr(rng, k, n, rng.integers(0, 70, k))
    for vt in (native.VAL_U32, native.VAL_U64):
        _check_product(native, engine, A, B, vt)


def test_wide_rows_use_several_windows(native, engine):
    """Dense-bin rows whose output spans more columns than one shared-memory window."""
    rng = np.random.default_rng(9)
    m, k, n = 40, 600, 200_000
    A = _random_csr(rng, m, k, rng.integers(200, 400, m))
    B = _random_csr(rng, k, n, np.full(k, 60))
    for vt in (native.VAL_U32, native.VAL_U64):
        _check_product(native, engine, A, B, vt)


def test_uint32_overflow_is_reported_and_uint64_is_exact(native, engine):
    import ctypes
    big = np.uint64(1 << 31)
    A = engine.upload(np.array([0, 2]), np.array([0, 1]), cols=2, val=np.array([big, big]), valtype=native.VAL_U32)
    B = engine.upload(np.array([0, 1, 2]), np.array([0, 0]), cols=1, val=np.array([1, 1]), valtype=native.VAL_U32)
    h = ctypes.c_void_p()
    rc = native.lib().rmcm_spgemm(engine._h, A._h, B._h, ctypes.byref(h))
    assert rc == native.EOVERFLOW
    native.lib().rmcm_mat_free(engine._h, h)
    A64 = engine.upload(np.array([0, 2]), np.array([0, 1]), cols=2, val=np.array([big, big]), valtype=native.VAL_U64)
    B64 = engine.upload(np.array([0, 1, 2]), np.array([0, 0]), cols=1, val=np.array([1, 1]), valtype=native.VAL_U64)
    C = engine.spgemm(A64, B64)
    assert C.download()[2].tolist() == [1 << 32]


def test_uint64_overflow_is_reported(native, engine):
    big = np.uint64(1 << 40)
    A = engine.upload(np.array([0, 1]), np.array([0]), cols=1, val=np.array([big]), valtype=native.VAL_U64)
    B = engine.upload(np.array([0, 1]), np.array([0]), cols=1, val=np.array([big]), valtype=native.VAL_U64)
    import ctypes
    h = ctypes.c_void_p()
    rc = native.lib().rmcm_spgemm(engine._h, A._h, B._h, ctypes.byref(h))
    assert rc == native.EOVERFLOW


def test_auto_mode_reruns_in_uint64(native):
    """K(64,64): an 8-matrix alternating chain has 64^7 = 2^42 paths per pair."""
    n = 64
    src = np.repeat(np.arange(n), n)
    dst = np.tile(np.arange(n), n)
    g = synth.SyntheticHIN("k64", [n, n], [synth.Relation(0, 1, 0, 1, src, dst)])
    eng = native.Engine(device=0, valtype=native.VAL_AUTO)
    hg = native.HeteroGraph.from_synthetic(eng, g)
    C, t, rc = eng.run_metapath(hg, "0-0-1-1-0-0-1-1-0-0-1-1-0-0-1-1-0")
    assert rc == native.OK and C.valtype == native.VAL_U64
    rp, col, val = C.download()
    assert C.nnz == n * n and set(val.tolist()) == {n ** 7}
    C.free()
    hg.close()
    eng.close()


def test_bad_arguments(native, engine):
    g = synth.tiny_dblp()
    hg = native.HeteroGraph.from_synthetic(engine, g)
    with pytest.raises(native.RmcmError) as e:
        engine.run_metapath(hg, "1-3")
    assert e.value.status == native.EINVAL
    with pytest.raises(native.RmcmError):
        engine.run_metapath(hg, "1-3-7-0-1")          # vertex type 7 is not in the graph
    A = engine.upload(np.array([0, 1]), np.array([0]), cols=3)
    B = engine.upload(np.array([0, 1, 1]), np.array([0]), cols=2)
    with pytest.raises(native.RmcmError) as e:
        engine.spgemm(A, B)
    assert e.value.status == native.EINVAL
    with pytest.raises(native.RmcmError) as e:
        engine.upload(np.array([0, 1]), np.array([5]), cols=3)
    assert e.value.status == native.EINVAL


def test_unsorted_upload_is_sorted(native, engine):
    M = engine.upload(np.array([0, 3]), np.array([4, 1, 2]), cols=5, val=np.array([7, 8, 9], np.uint64),
                      valtype=native.VAL_U64)
    rp, col, val = M.download()
    assert col.tolist() == [1, 2, 4] and val.tolist() == [8, 9, 7]


def test_memory_budget_is_enforced(native):
    eng = native.Engine(device=0, mem_budget_bytes=4 << 20)
    g = synth.dblp_like(n_a=3000, n_p=6000, n_v=20, seed=7)
    hg = native.HeteroGraph.from_synthetic(eng, g)
    with pytest.raises(native.RmcmError) as e:
        eng.run_metapath(hg, "0-0-1-3-0")             # 8.5M nnz result does not fit in 4 MB
    assert e.value.status == native.ENOMEM
    hg.close()
    eng.close()


def test_cli_output_line(native, tmp_path):
    g = synth.tiny_dblp()
    files = g.write_text(str(tmp_path))
    out = tmp_path / "out.txt"
    r = subprocess.run([native.CLI_PATH, "4", "1", files["graph"], files["vertex"], files["edge"],
                        files["metapaths"], str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = out.read_text().splitlines()
    assert [ln.split()[0] for ln in lines] == g.metapaths
    assert [int(ln.split()[1]) for ln in lines] == [7, 9, 14, 1, 4]
    for ln in lines:
        parts = ln.split()
        assert len(parts) == 6
        [float(x) for x in parts[2:]]


def test_graph_outliving_its_handle_is_safe(native):
    """Destroying a handle first orphans its graphs; freeing them later is host-only."""
    eng = native.Engine(device=0)
    hg = native.HeteroGraph.from_synthetic(eng, synth.tiny_dblp())
    C, _, _ = eng.run_metapath(hg, "1-3-0-0-1")
    C.free()
    eng.close()
    hg.close()


def test_explicit_zero_values_keep_the_structure(native, engine):
    """A stored 0 is still an entry: the structure is the Boolean product's."""
    rng = np.random.default_rng(12)
    A = _random_csr(rng, 200, 300, rng.integers(1, 80, 200), vmax=3)
    B = _random_csr(rng, 300, 3000, rng.integers(1, 200, 300), vmax=3)
    A.data[::5] = 0                       # explicit zeros, kept in the CSR
    A.sort_indices(); B.sort_indices()
    pattern = (sp.csr_matrix((np.ones_like(A.data), A.indices, A.indptr), A.shape)
               @ sp.csr_matrix((np.ones_like(B.data), B.indices, B.indptr), B.shape)).tocsr()
    pattern.sort_indices()
    dense = A.toarray() @ B.toarray()
    for vt in (native.VAL_U32, native.VAL_U64):
        Am = engine.upload(A.indptr, A.indices, cols=A.shape[1], val=A.data.astype(np.uint64), valtype=vt)
        Bm = engine.upload(B.indptr, B.indices, cols=B.shape[1], val=B.data.astype(np.uint64), valtype=vt)
        rp, col, val = engine.spgemm(Am, Bm).download()
        assert np.array_equal(rp, pattern.indptr) and np.array_equal(col, pattern.indices)
        rows = np.repeat(np.arange(A.shape[0]), np.diff(rp))
        assert np.array_equal(val.astype(np.int64), dense[rows, col].astype(np.int64))


def test_fully_dense_b_rows_use_the_register_path(native, engine):
    """B rows covering every column of a narrow window (plus some that do not)."""
    rng = np.random.default_rng(21)
    m, k, n = 300, 500, 1500
    A = _random_csr(rng, m, k, rng.integers(1, 120, m), vmax=5)
    rows_nnz = np.where(rng.random(k) < 0.6, n, rng.integers(1, n, k))
    B = _random_csr(rng, k, n, rows_nnz, vmax=5)
    for vt in (native.VAL_U32, native.VAL_U64):
        _check_product(native, engine, A, B, vt)


def test_full_length_rows_with_repeats_are_not_dense(native, engine):
    """A row as long as the window but with a repeated column does not cover it."""
    Bd = np.array([[2, 1, 1, 0]] * 40, np.uint64)          # 4 columns, column 3 empty
    rp = np.arange(0, 4 * 40 + 1, 4, dtype=np.int64)
    col = np.tile(np.array([0, 0, 1, 2], np.int32), 40)     # column 0 listed twice
    val = np.tile(np.array([1, 1, 1, 1], np.uint64), 40)
    B = engine.upload(rp, col, cols=4, val=val, valtype=native.VAL_U32)
    arp = np.array([0, 40], np.int64)
    A = engine.upload(arp, np.arange(40, dtype=np.int32), cols=40, valtype=native.VAL_U32)
    C = engine.spgemm(A, B)
    rpc, colc, valc = C.download()
    assert colc.tolist() == [0, 1, 2] and valc.tolist() == [80, 40, 40]


def test_dense_register_path_detects_overflow(native, engine):
    import ctypes
    k, n = 64, 1000
    big = np.uint64(1 << 27)
    rp = np.arange(0, k * n + 1, n, dtype=np.int64)
    col = np.tile(np.arange(n, dtype=np.int32), k)
    B = engine.upload(rp, col, cols=n, val=np.full(k * n, big, np.uint64), valtype=native.VAL_U32)
    A = engine.upload(np.array([0, k], np.int64), np.arange(k, dtype=np.int32), cols=k,
                      val=np.full(k, 2, np.uint64), valtype=native.VAL_U32)
    h = ctypes.c_void_p()
    rc = native.lib().rmcm_spgemm(engine._h, A._h, B._h, ctypes.byref(h))
    assert rc == native.EOVERFLOW            # 64 * 2 * 2^27 = 2^34 per column
    native.lib().rmcm_mat_free(engine._h, h)
    B64 = engine.upload(rp, col, cols=n, val=np.full(k * n, big, np.uint64), valtype=native.VAL_U64)
    A64 = engine.upload(np.array([0, k], np.int64), np.arange(k, dtype=np.int32), cols=k,
                        val=np.full(k, 2, np.uint64), valtype=native.VAL_U64)
    C = engine.spgemm(A64, B64)
    assert set(C.download()[2].tolist()) == {1 << 34}


@pytest.mark.parametrize("n", [60_000, 61_441, 65_535, 1 << 20])
def test_rank_bin_for_wide_rows(native, engine, n):
    """Rows wider than a dense window (up to 2^20 columns) with > 4096 products;
    widths one past and one short of a 4096-column group, with entries on the
    first and last columns of groups and of the row."""
    rng = np.random.default_rng(31)
    m, k = 40, 400
    A = _random_csr(rng, m, k, rng.integers(100, 300, m), vmax=4)
    B = _random_csr(rng, k, n, rng.integers(20, 100, k), vmax=4).tolil()
    edges = [c for g in range(4096, n, 4096) for c in (g - 1, g)] + [0, n - 1]
    for i, c in enumerate(edges):
        B[(7 * i) % k, c] = 1 + i % 4
    B = B.tocsr()
    for vt in (native.VAL_U32, native.VAL_U64):
        _check_product(native, engine, A, B, vt)


def test_rank_bin_short_and_long_wide_rows(native, engine):
    """2^20-column rows in one rank launch: most with ~10K entries, two with
    more than 30K; uint32 and uint64 match scipy."""
    rng = np.random.default_rng(37)
    m, k, n = 30, 3000, 1 << 20
    a_nnz = rng.integers(150, 250, m)
    a_nnz[5] = 700
    a_nnz[17] = 900
    A = _random_csr(rng, m, k, a_nnz, vmax=3)
    B = _random_csr(rng, k, n, rng.integers(40, 80, k), vmax=3)
    ref = (A @ B).tocsr()
    assert np.diff(ref.indptr).max() > 30_000 and np.median(np.diff(ref.indptr)) < 15_000
    for vt in (native.VAL_U32, native.VAL_U64):
        _check_product(native, engine, A, B, vt)


def test_rank_bin_detects_overflow(native, engine):
    import ctypes
    rng = np.random.default_rng(32)
    k, n = 200, 300_000
    B = _random_csr(rng, k, n, np.full(k, 50), vmax=1)
    B.data[:] = 1 << 26
    rp = np.array([0, k], np.int64)
    acol = np.arange(k, dtype=np.int32)
    for vt, expect in ((native.VAL_U32, native.EOVERFLOW), (native.VAL_U64, native.OK)):
        Bm = engine.upload(B.indptr, B.indices, cols=n, val=B.data.astype(np.uint64), valtype=vt)
        Am = engine.upload(rp, acol, cols=k, val=np.full(k, 64, np.uint64), valtype=vt)
        h = ctypes.c_void_p()
        rc = native.lib().rmcm_spgemm(engine._h, Am._h, Bm._h, ctypes.byref(h))
        assert rc == expect
        if vt == native.VAL_U64:
            C = native.Matrix(engine, h.value)
            ref = (sp.csr_matrix((np.full(k, 64, np.int64), acol, rp), shape=(1, k)) @ B.astype(np.int64)).tocsr()
            ref.sort_indices()
            got = C.download()
            assert np.array_equal(got[1], ref.indices) and np.array_equal(got[2].astype(np.int64), ref.data)
        else:
            native.lib().rmcm_mat_free(engine._h, h)


@pytest.mark.parametrize("mode", ["l2r", "dense"])
def test_ablation_orders_give_the_same_result(native, mode):
    from helpers import load_fixture, make_graph
    fx = load_fixture("dblp_small")
    eng = native.Engine(device=0)
    hg = native.HeteroGraph.from_synthetic(eng, make_graph(fx))
    refs = {}
    for rec in fx["paths"][:5]:
        C, t, _ = eng.run_metapath(hg, rec["metapath"])
        refs[rec["metapath"]] = C.download()
        C.free()
    eng.set_order_mode(native.ORDER_L2R if mode == "l2r" else native.ORDER_DENSE)
    for rec in fx["paths"][:5]:
        C, t, _ = eng.run_metapath(hg, rec["metapath"])
        got = C.download()
        C.free()
        for a, b in zip(refs[rec["metapath"]], got):
            assert np.array_equal(a, b), rec["metapath"]
        if rec["len"] >= 2:
            assert t["es_s"] == 0.0
    hg.close()
    eng.close()


def test_graph_cache_roundtrip(native, engine, tmp_path):
    g = synth.dblp_like(n_a=3000, n_p=6000, n_v=20, seed=7)
    hg = native.HeteroGraph.from_synthetic(engine, g)
    path = str(tmp_path / "g.bin")
    hg.save(path)
    hg2 = native.HeteroGraph.load(engine, path)
    assert hg2.info() == hg.info()
    a, _, _ = engine.run_metapath(hg, "1-3-0-1-2-4-0-0-1")
    b, _, _ = engine.run_metapath(hg2, "1-3-0-1-2-4-0-0-1")
    for x, y in zip(a.download(), b.download()):
        assert np.array_equal(x, y)
    assert np.array_equal(hg2.global_ids(1), np.arange(6000, 9000))


def test_cli_flags(native, tmp_path):
    g = synth.tiny_dblp()
    files = g.write_text(str(tmp_path))
    run = lambda *extra: subprocess.run([native.CLI_PATH, "4", "1", files["graph"], files["vertex"], files["edge"],
                                         files["metapaths"], *extra], capture_output=True, text=True, timeout=300)
    # estimator only: accuracy/res line format
    est = tmp_path / "est.txt"
    r = run(str(est), "--estimate-only")
    assert r.returncode == 0, r.stderr
    lines = est.read_text().splitlines()
    assert [ln.split()[0] for ln in lines] == g.metapaths and all(len(ln.split()) == 2 for ln in lines)
    # cache + result sinks
    cache = tmp_path / "g.bin"
    res_dir = tmp_path / "res"
    cnt_dir = tmp_path / "cnt"
    res_dir.mkdir()
    cnt_dir.mkdir()
    for _ in range(2):   # second run reads the cache
        out = tmp_path / "out.txt"
        r = run(str(out), f"--cache={cache}", f"--save-result={res_dir}", f"--row-counts={cnt_dir}", "--order=l2r")
        assert r.returncode == 0, r.stderr
        assert cache.exists()
    rows, cols, rp, col, val = native.read_csr(str(res_dir / "1-3-0-0-1.csr"))
    assert (rows, cols) == (3, 3) and int(rp[-1]) == 7 and set(val.tolist()) <= {1, 2}
    cnt = (cnt_dir / "1-3-0-0-1.cnt").read_text().split()
    assert cnt == ["4", "3", "5", "2", "6", "2"]        # global author ids 4..6 and their row sizes


def test_heavy_dense_rows_are_split_over_ctas(native, engine):
    """One row with ~4.7M products (above the split threshold) among light
    rows: the heavy row goes through the split kernels, the rest through the
    dense bin; both must match scipy, in uint32 and uint64."""
    rng = np.random.default_rng(31)
    m, k, n = 40, 3000, 1800
    a_nnz = rng.integers(1, 30, m)
    a_nnz[7] = k                         # the heavy row: every B row
    A = _random_csr(rng, m, k, a_nnz, vmax=3)
    B = _random_csr(rng, k, n, rng.integers(1500, 1800, k), vmax=3)
    for vt in (native.VAL_U32, native.VAL_U64):
        eng = native.Engine(device=0)
        eng.set_profiling(1)
        _check_product(native, eng, A, B, vt)
        st = eng.product_stats()[0]
        assert st["flops"] > (1 << 22) and st["bin_rows"][4] > 0
        eng.close()


def test_split_rows_replay_in_a_batch(native):
    """A star-shaped relation gives one vertex millions of two-step paths; the
    batch replays its split product exactly."""
    rng = np.random.default_rng(32)
    n0, n1, n2 = 4, 2600, 1800
    src01 = np.concatenate([np.zeros(n1, np.int64), rng.integers(1, n0, 50)])
    dst01 = np.concatenate([np.arange(n1), rng.integers(0, n1, 50)])
    deg = rng.integers(1700, 1790, n1)
    src12 = np.repeat(np.arange(n1), deg)
    dst12 = np.concatenate([rng.choice(n2, d, replace=False) for d in deg])
    src01, dst01 = synth.dedup_pairs_keep_order(src01, dst01, n1)
    g = synth.SyntheticHIN("star", [n0, n1, n2], [synth.Relation(0, 1, 0, 1, src01, dst01),
                                                  synth.Relation(1, 2, 2, 3, src12, dst12)])
    eng = native.Engine(device=0)
    hg = native.HeteroGraph.from_synthetic(eng, g)
    paths = ["0-0-1-2-2", "0-0-1-2-2-3-1", "2-3-1-1-0-0-1-2-2"]
    plain = []
    for mp in paths:
        C, _, rc = eng.run_metapath(hg, mp)
        plain.append(eng.digest(C))
        C.free()
    b = eng.batch(hg, paths, lanes=2)
    for _ in range(2):
        nnz, dig, _ = b.run()
        assert [(int(a), int(x)) for a, x in zip(nnz, dig)] == plain
    b.free()
    hg.close()
    eng.close()


def test_long_rows_are_analysed_by_the_whole_grid(native, engine):
    """A rows longer than the per-warp analysis limit (16384 entries): their
    products and count bounds come from grid-wide partial sums."""
    rng = np.random.default_rng(33)
    m, k, n = 6, 60000, 700
    a_nnz = np.array([3, 40000, 10, 20000, 0, 5])
    A = _random_csr(rng, m, k, a_nnz, vmax=4)
    B = _random_csr(rng, k, n, rng.integers(0, 6, k), vmax=4)
    for vt in (native.VAL_U32, native.VAL_U64):
        _check_product(native, engine, A, B, vt)


def test_estimator_long_rows_match_the_oracle(native, oracle_mod):
    """Rows of more than 4096 entries get a whole CTA in the estimator; the
    estimates stay within 1e-9 of the oracle's and are reproducible."""
    rng = np.random.default_rng(34)
    n0, n1, n2 = 3, 9000, 500
    src01 = np.concatenate([np.zeros(6000, np.int64), np.full(5000, 1), rng.integers(0, n0, 200)])
    dst01 = np.concatenate([rng.choice(n1, 6000, replace=False), rng.choice(n1, 5000, replace=False),
                            rng.integers(0, n1, 200)])
    src01, dst01 = synth.dedup_pairs_keep_order(src01, dst01, n1)
    src12 = rng.integers(0, n1, 30000)
    dst12 = rng.integers(0, n2, 30000)
    src12, dst12 = synth.dedup_pairs_keep_order(src12, dst12, n2)
    g = synth.SyntheticHIN("long_est", [n0, n1, n2], [synth.Relation(0, 1, 0, 1, src01, dst01),
                                                      synth.Relation(1, 2, 2, 3, src12, dst12)])
    eng = native.Engine(device=0)
    hg = native.HeteroGraph.from_synthetic(eng, g)
    og = oracle_mod.OracleGraph.from_synthetic(g)
    for mp in ["0-0-1-2-2-3-1-1-0", "0-0-1-2-2", "2-3-1-1-0-0-1-2-2"]:
        c1 = eng.estimate(hg.leaves(mp))
        c2 = eng.estimate(hg.leaves(mp))
        assert np.array_equal(c1, c2)
        want = og.estimate(mp, threads=1)
        nz = want != 0
        assert np.array_equal(c1[~nz], want[~nz])
        assert (np.abs(c1[nz] - want[nz]) / np.abs(want[nz])).max(initial=0) <= 1e-9
    og.close()
    hg.close()
    eng.close()


def test_async_download_and_deferred_free(native, engine):
    """rmcm_mat_download_async gives the same arrays as the synchronous copy,
    even when the matrix is freed before the transfers are waited for."""
    g = synth.tiny_dblp()
    hg = native.HeteroGraph.from_synthetic(engine, g)
    want = []
    outs = []
    for mp in ["1-3-0-1-2-4-0-0-1", "1-3-0-0-1"]:
        C, _, _ = engine.run_metapath(hg, mp)
        want.append(C.download())
        rp = np.zeros(C.shape[0] + 1, np.int64)
        col = np.zeros(max(C.nnz, 1), np.int32)
        val = np.zeros(max(C.nnz, 1), np.uint64 if C.valtype == native.VAL_U64 else np.uint32)
        engine.download_async(C, rp.ctypes.data, col.ctypes.data, val.ctypes.data)
        C.free()                                  # released once the copy has landed
        outs.append((rp, col, val))
    engine.transfers_wait()
    for (rp, col, val), (wrp, wcol, wval) in zip(outs, want):
        assert np.array_equal(rp, wrp) and np.array_equal(col[:wcol.size], wcol)
        assert np.array_equal(val[:wval.size].astype(np.uint64), wval.astype(np.uint64))
    hg.close()


def test_split_rows_with_full_width_b_rows(native):
    """Heavy rows split over CTAs whose B rows cover every column take the
    register path inside the split kernel; uint32 and uint64 match scipy."""
    rng = np.random.default_rng(35)
    m, k, n = 24, 2600, 2000
    a_nnz = rng.integers(1, 40, m)
    a_nnz[5] = k
    a_nnz[17] = 2000
    A = _random_csr(rng, m, k, a_nnz, vmax=3)
    rows_nnz = np.where(rng.random(k) < 0.6, n, rng.integers(1000, n, k))
    B = _random_csr(rng, k, n, rows_nnz, vmax=3)
    for vt in (native.VAL_U32, native.VAL_U64):
        eng = native.Engine(device=0)
        _check_product(native, eng, A, B, vt)
        eng.close()


def test_heavy_rank_rows_are_split_over_ctas(native):
    """Rows wider than a dense window (rank bin) with millions of products:
    the heavy rows are split over CTAs (global bitmap + ranks); the light ones
    stay in the rank kernel; uint32 and uint64 match scipy."""
    rng = np.random.default_rng(36)
    m, k, n = 12, 21000, 60000
    a_nnz = rng.integers(200, 400, m)
    a_nnz[3] = 20000
    a_nnz[9] = 15000
    A = _random_csr(rng, m, k, a_nnz, vmax=3)
    B = _random_csr(rng, k, n, rng.integers(60, 140, k), vmax=3)
    for vt in (native.VAL_U32, native.VAL_U64):
        eng = native.Engine(device=0)
        eng.set_profiling(1)
        _check_product(native, eng, A, B, vt)
        st = eng.product_stats()[0]
        assert st["bin_rows"][5] > 0
        eng.close()


def test_matrices_of_one_handle_feed_another_after_synchronize(native, engine):
    """A loader handle uploads a chain's leaves; after rmcm_synchronize the
    compute handle multiplies them: same result as with its own uploads."""
    g = synth.tiny_dblp()
    hg = native.HeteroGraph.from_synthetic(engine, g)
    mp = "1-3-0-1-2-4-0-0-1"
    want, _, _ = engine.run_metapath(hg, mp)
    want_arrays = want.download()
    want.free()
    loader = native.Engine(device=0)
    mats = []
    for leaf in hg.leaves(mp):
        rp, col, _ = leaf.download(values=False)
        mats.append(loader.upload(rp, col, cols=leaf.shape[1]))
    loader.synchronize()
    C, _, rc = engine.chain(mats)
    got = C.download()
    C.free()
    for a, b in zip(got, want_arrays):
        assert np.array_equal(a, b)
    for m in mats:
        m.free()
    loader.close()
    hg.close()


def _heavy_reuse(rng, m, k, n, big=None):
    """A (m x k) with every row long, B (k x n) rows of 40..n entries: the
    product has hundreds of multiply-adds per entry of B (B is packed for the
    dense bin).  ``big``: one entry per B row set to this value."""
    A = _random_csr(rng, m, k, rng.integers(k // 2, k + 1, m), vmax=5)
    B = _random_csr(rng, k, n, rng.integers(40, n + 1, k), vmax=5).tocsr()
    if big is not None:
        B.data[B.indptr[:-1][np.diff(B.indptr) > 0]] = big
    return A, B


@pytest.mark.parametrize("n", [1500, 2047, 2048, 2049])
def test_packed_b_for_heavy_reuse(native, engine, n):
    """Dense rows whose B entries are reused many times read a packed copy of
    B ((value << column bits) | column, rows reordered by shared-memory bank);
    column counts at the edges of the column bits."""
    rng = np.random.default_rng(40 + n)
    A, B = _heavy_reuse(rng, 300, 60, n)
    for vt in (native.VAL_U32, native.VAL_U64):
        _check_product(native, engine, A, B, vt)


def test_values_too_large_to_pack(native, engine):
    """A B value at 2^21 + 5 does not fit beside 11 column bits: B stays
    unpacked and the product is still exact."""
    rng = np.random.default_rng(44)
    A, B = _heavy_reuse(rng, 300, 60, 1500, big=(1 << 21) + 5)
    A.data[:] = 1
    _check_product(native, engine, A, B, native.VAL_U32)


def test_packed_b_replays_in_a_batch(native):
    """A meta-path whose product packs B gives the same (nnz, digest) when
    replayed from a batch's CUDA graph."""
    rng = np.random.default_rng(45)
    nx, ny, nz = 400, 60, 1500
    xs = np.repeat(np.arange(nx), 45)
    xy = rng.integers(0, ny, xs.size)
    src01, dst01 = synth.dedup_pairs_keep_order(xs, xy, ny)
    ys = np.repeat(np.arange(ny), 700)
    yz = rng.integers(0, nz, ys.size)
    src12, dst12 = synth.dedup_pairs_keep_order(ys, yz, nz)
    g = synth.SyntheticHIN("reuse", [nx, ny, nz], [synth.Relation(0, 1, 0, 1, src01, dst01),
                                                   synth.Relation(1, 2, 2, 3, src12, dst12)])
    eng = native.Engine(device=0)
    hg = native.HeteroGraph.from_synthetic(eng, g)
    paths = ["0-0-1-2-2", "2-3-1-1-0-0-1-2-2"]
    plain = []
    for mp in paths:
        C, _, _ = eng.run_metapath(hg, mp)
        plain.append(eng.digest(C))
        C.free()
    b = eng.batch(hg, paths, lanes=2)
    for _ in range(2):
        nnz, dig, _ = b.run()
        assert [(int(a), int(x)) for a, x in zip(nnz, dig)] == plain
    b.free()
    hg.close()
    eng.close()


@pytest.mark.parametrize("n", [300, 2000, 2048, 2049])
def test_warp_bin_rows(native, n):
    """Rows of an output at most 2048 columns wide with 33..2048 products get
    a warp each with its own window; equal to scipy in uint32 and uint64, and
    to the same product with the warp bin turned off.  A 2049-column output
    never uses it."""
    rng = np.random.default_rng(50 + n)
    m, k = 1500, 3000
    A = _random_csr(rng, m, k, rng.integers(0, 24, m), vmax=5)
    B = _random_csr(rng, k, n, rng.integers(0, min(n, 150), k), vmax=5)
    for vt in (native.VAL_U32, native.VAL_U64):
        eng = native.Engine(device=0)
        _check_product(native, eng, A, B, vt)
        eng.set_tuning(warp_max_flops=0)
        _check_product(native, eng, A, B, vt)
        eng.close()


def test_warp_bin_risky_rows(native, engine):
    """Rows whose count bound exceeds uint32 take the checked adds of the warp
    bin: exact when no entry overflows, EOVERFLOW (and exact in uint64) when
    one does."""
    rng = np.random.default_rng(60)
    m, k, n = 400, 800, 1000
    A = _random_csr(rng, m, k, rng.integers(1, 20, m), vmax=1)
    B = _random_csr(rng, k, n, rng.integers(50, 100, k), vmax=1).tocsr()
    B.data[:] = rng.integers(1 << 26, 1 << 27, B.nnz)
    _check_product(native, engine, A, B, native.VAL_U32)
    # 33 products (warp bin) all on column 0 at 2^27: 33 * 2^27 > 2^32
    A2 = A.tolil()
    A2[0, :] = 0
    A2[0, :33] = 1
    A2 = A2.tocsr()
    B2 = B.tolil()
    B2[:33, :] = 0
    B2[:33, 0] = 1 << 27
    B2 = B2.tocsr()
    B2.eliminate_zeros()
    import ctypes
    Am = engine.upload(A2.indptr, A2.indices, cols=k, val=A2.data.astype(np.uint64), valtype=native.VAL_U32)
    Bm = engine.upload(B2.indptr, B2.indices, cols=n, val=B2.data.astype(np.uint64), valtype=native.VAL_U32)
    h = ctypes.c_void_p()
    assert native.lib().rmcm_spgemm(engine._h, Am._h, Bm._h, ctypes.byref(h)) == native.EOVERFLOW
    native.lib().rmcm_mat_free(engine._h, h)
    _check_product(native, engine, A2, B2, native.VAL_U64)


def _heavy_inner(rng, m, k, n, nheavy, bbig=None):
    """A (m x k) with `nheavy` nearly full columns and sparse others, B (k x n)
    whose rows for those columns are half full: the product's heavy inner
    indices go to the tensor-core GEMM, the rest stays sparse.  ``bbig``: a
    few B values that need more than one limb."""
    dense_a = (rng.random((m, nheavy)) < 0.8) * rng.integers(1, 4, (m, nheavy))
    light_a = sp.random(m, k - nheavy, density=0.03, random_state=rng, format="csr")
    light_a.data[:] = rng.integers(1, 4, light_a.nnz)
    A = sp.hstack([sp.csr_matrix(dense_a), light_a]).tocsr()
    dense_b = (rng.random((nheavy, n)) < 0.5) * rng.integers(1, 4, (nheavy, n))
    light_b = sp.random(k - nheavy, n, density=0.02, random_state=rng, format="csr")
    light_b.data[:] = rng.integers(1, 4, light_b.nnz)
    B = sp.vstack([sp.csr_matrix(dense_b), light_b]).tocsr()
    if bbig is not None:
        B = B.tolil()
        for u in range(0, nheavy, 7):
            B[u, (u * 13) % n] = bbig
        B = B.tocsr()
    A.eliminate_zeros()
    B.eliminate_zeros()
    return A, B


@pytest.mark.parametrize("bbig,limbs", [(None, 1), (5000, 2), (200000, 2), (5000000, 3)])
def test_tensor_core_part_of_dense_rows(native, bbig, limbs):
    """Heavy inner indices multiplied as FP16 GEMMs on the tensor cores with
    FP32 accumulation (B split into one to three limbs when its values are
    wide, the limbs summed by the GEMM's epilogue): the product equals scipy's
    and the same product with the GEMM turned off, bit for bit."""
    rng = np.random.default_rng(70 if bbig is None else bbig)
    A, B = _heavy_inner(rng, 1200, 2500, 1500, 300, bbig)
    eng = native.Engine(device=0)
    eng.set_tuning(gemm_min_mflops=0)
    eng.set_profiling(1)
    _check_product(native, eng, A, B, native.VAL_U32)
    st = eng.product_stats()[-1]
    assert st["gemm_inner"] >= 250 and st["gemm_limbs"] == limbs
    eng.set_tuning(gemm_inv_density=0)
    _check_product(native, eng, A, B, native.VAL_U32)
    assert eng.product_stats()[-1]["gemm_inner"] == 0
    eng.close()


def test_tensor_core_part_in_a_chain_and_batch(native):
    """A meta-path whose product takes the tensor-core part gives the same
    (nnz, digest) run plainly (GEMM) and replayed from a batch (no GEMM)."""
    rng = np.random.default_rng(71)
    nx, ny, nz = 800, 1500, 1200
    heavy = 200
    xs, ys = [], []
    for x in range(nx):
        cols = np.concatenate([np.nonzero(rng.random(heavy) < 0.8)[0],
                               heavy + rng.choice(ny - heavy, 40, replace=False)])
        xs += [x] * cols.size
        ys += cols.tolist()
    src01, dst01 = synth.dedup_pairs_keep_order(np.array(xs), np.array(ys), ny)
    ys2, zs = [], []
    for y in range(ny):
        k = nz // 2 if y < heavy else 20
        cols = rng.choice(nz, k, replace=False)
        ys2 += [y] * k
        zs += cols.tolist()
    src12, dst12 = synth.dedup_pairs_keep_order(np.array(ys2), np.array(zs), nz)
    g = synth.SyntheticHIN("gemm", [nx, ny, nz], [synth.Relation(0, 1, 0, 1, src01, dst01),
                                                  synth.Relation(1, 2, 2, 3, src12, dst12)])
    eng = native.Engine(device=0)
    eng.set_tuning(gemm_min_mflops=0)
    eng.set_profiling(1)
    hg = native.HeteroGraph.from_synthetic(eng, g)
    paths = ["0-0-1-2-2"]
    C, _, _ = eng.run_metapath(hg, paths[0])
    assert eng.product_stats()[-1]["gemm_inner"] >= 150
    plain = [eng.digest(C)]
    C.free()
    eng.set_tuning(gemm_inv_density=0)
    C, _, _ = eng.run_metapath(hg, paths[0])
    assert eng.digest(C) == plain[0]
    C.free()
    eng.set_tuning(gemm_inv_density=256)
    b = eng.batch(hg, paths, lanes=1)
    nnz, dig, _ = b.run()
    assert [(int(a), int(x)) for a, x in zip(nnz, dig)] == plain
    b.free()
    hg.close()
    eng.close()


def test_tensor_core_part_uint64(native):
    """uint64 products: A and B both split into FP16 limbs and the heavy
    indices into chunks (every partial sum <= 2^24); equal to scipy's int64
    product and to the same product with the GEMM turned off."""
    rng = np.random.default_rng(72)
    A, B = _heavy_inner(rng, 1200, 2500, 1500, 300, bbig=200000)
    A = A.tocsr()
    A.data = A.data * 1000
    eng = native.Engine(device=0)
    eng.set_tuning(gemm_min_mflops=0)
    eng.set_profiling(1)
    _check_product(native, eng, A, B, native.VAL_U64)
    st = eng.product_stats()[-1]
    assert st["gemm_inner"] >= 250 and st["gemm_limbs"] >= 4
    eng.set_tuning(gemm_inv_density=0)
    _check_product(native, eng, A, B, native.VAL_U64)
    assert eng.product_stats()[-1]["gemm_inner"] == 0
    eng.close()


def _plant_wide_a(A, heavy, value=3000):
    """Every third row of A gets `value` (> 2047: two FP16 limbs) at one of
    the heavy inner indices."""
    A = A.tolil()
    for r in range(0, A.shape[0], 3):
        A[r, r % heavy] = value
    return A.tocsr()


def test_tensor_core_part_uint32_limbs_of_a(native):
    """A uint32 product whose heavy A values do not fit one FP16 limb (some
    are 3000): the GEMM splits A into limbs too (2 x 1 limb pairs) and the
    seeds are summed modulo 2^32 like the counters.  Equal to scipy and to
    the GEMM off, bit for bit."""
    rng = np.random.default_rng(74)
    A, B = _heavy_inner(rng, 1200, 2500, 1500, 300)
    A = _plant_wide_a(A, 300)
    eng = native.Engine(device=0)
    eng.set_tuning(gemm_min_mflops=0)
    eng.set_profiling(1)
    _check_product(native, eng, A, B, native.VAL_U32)
    st = eng.product_stats()[-1]
    assert st["gemm_inner"] >= 250 and st["gemm_limbs"] == 2
    eng.set_tuning(gemm_inv_density=0)
    _check_product(native, eng, A, B, native.VAL_U32)
    assert eng.product_stats()[-1]["gemm_inner"] == 0
    eng.close()


@pytest.mark.parametrize("wide_a", [False, True])
def test_tensor_core_part_with_skewed_rows(native, wide_a):
    """A uint32 product with one row far heavier than a fair share: the GEMM
    takes the heavy inner indices of every row, and the heavy row's light
    entries (~1.5M products) are split over CTAs whose sums are added to the
    row's GEMM seeds (one limb of A, or two with ``wide_a``).  Equal to scipy
    and to the GEMM off, bit for bit."""
    rng = np.random.default_rng(73)
    m, heavy, light, n = 600, 300, 20000, 1500
    dense_a = (rng.random((m, heavy)) < 0.8) * rng.integers(1, 4, (m, heavy))
    light_a = sp.random(m, light, density=0.03, random_state=rng, format="lil")
    light_a[7, :] = 1                                   # the skewed row: every light index
    light_a = light_a.tocsr()
    light_a.data[:] = rng.integers(1, 4, light_a.nnz)
    A = sp.hstack([sp.csr_matrix(dense_a), light_a]).tocsr()
    if wide_a:
        A = _plant_wide_a(A, heavy)
    dense_b = (rng.random((heavy, n)) < 0.5) * rng.integers(1, 4, (heavy, n))
    light_b = sp.random(light, n, density=0.05, random_state=rng, format="csr")
    light_b.data[:] = rng.integers(1, 4, light_b.nnz)
    B = sp.vstack([sp.csr_matrix(dense_b), light_b]).tocsr()
    A.eliminate_zeros()
    B.eliminate_zeros()
    eng = native.Engine(device=0)
    eng.set_tuning(gemm_min_mflops=0)
    eng.set_profiling(1)
    _check_product(native, eng, A, B, native.VAL_U32)
    st = eng.product_stats()[-1]
    assert st["gemm_inner"] >= 250 and st["bin_rows"][4] == m
    assert st["gemm_limbs"] == (2 if wide_a else 1)
    eng.set_tuning(gemm_inv_density=0)
    _check_product(native, eng, A, B, native.VAL_U32)
    assert eng.product_stats()[-1]["gemm_inner"] == 0
    eng.close()


@pytest.mark.parametrize("m,n,heavy", [(256, 90, 300), (129, 1030, 200), (640, 384, 513), (131, 2100, 64)])
def test_tensor_core_part_tile_edges(native, m, n, heavy):
    """The tensor-core GEMM's 128 x 128 output tiles and 64-wide K blocks at
    their edges: rows and columns that fill a tile exactly, fall one short or
    one over, fewer columns than a tile and than a multiple of 8, and heavy
    index counts just past a K block.  Equal to scipy and to the GEMM off."""
    rng = np.random.default_rng(m * 7919 + n)
    A, B = _heavy_inner(rng, m, heavy + 900, n, heavy)
    eng = native.Engine(device=0)
    eng.set_tuning(gemm_min_mflops=0)
    eng.set_profiling(1)
    _check_product(native, eng, A, B, native.VAL_U32)
    assert eng.product_stats()[-1]["gemm_inner"] >= heavy // 2
    _check_product(native, eng, A, B, native.VAL_U64)
    assert eng.product_stats()[-1]["gemm_inner"] >= heavy // 2
    eng.set_tuning(gemm_inv_density=0)
    _check_product(native, eng, A, B, native.VAL_U32)
    assert eng.product_stats()[-1]["gemm_inner"] == 0
    eng.close()


@pytest.mark.parametrize("vt,m,n,heavy,scale_a,bbig", [
    ("u32", 300, 500, 1100, 1, None),        # 4 tiles of 256 x 256, 18 K blocks: every tile in two units
    ("u64", 1200, 1500, 600, 1000, 200000),  # two A and two B limbs, 10 chunks: units span several groups
])
def test_tensor_core_part_split_units(native, vt, m, n, heavy, scale_a, bbig):
    """Fewer output tiles than SMs: the tensor-core GEMM splits each tile's
    K blocks over several CTAs that add their parts into the seeds with
    atomics.  Equal to scipy and to the GEMM off, bit for bit."""
    rng = np.random.default_rng(m + n + heavy)
    A, B = _heavy_inner(rng, m, heavy + 1500, n, heavy, bbig)
    A = A.tocsr()
    A.data = A.data * scale_a
    val = native.VAL_U32 if vt == "u32" else native.VAL_U64
    eng = native.Engine(device=0)
    eng.set_tuning(gemm_min_mflops=0)
    eng.set_profiling(1)
    for _ in range(2):
        _check_product(native, eng, A, B, val)
        assert eng.product_stats()[-1]["gemm_inner"] >= heavy // 2
    eng.set_tuning(gemm_inv_density=0)
    _check_product(native, eng, A, B, val)
    assert eng.product_stats()[-1]["gemm_inner"] == 0
    eng.close()
