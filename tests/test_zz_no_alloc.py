"""The estimator entry point that allocates nothing, through the C ABI.

rmcm_estimate_noalloc exists for callers that may not allocate device memory
when they need an estimate (a framework that owns all device memory in its
own pool, a serving loop that forbids allocation after start-up).  They hand
over the chain as device CSR arrays they own; the entry point keeps its
temporaries in a fixed device array built into the library.  These tests
give it the same chains as the allocating entry point, rmcm_estimate, twice
in a row (the second call reuses the array the first one left behind) and
check every estimate against the allocating one within the estimator
tolerance of the parity tests, 1e-9 relative; a chain with a row longer than
the allocating path's long-row threshold is also checked against the CPU
oracle.  They check that a call after the first one leaves the device's free
memory unchanged, that a call on a non-default stream gives the same
estimates, and that chains too large for the fixed array are refused before
anything runs.  The file is collected last so that a failure here cannot
hide the other tests' results.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import load_fixture, make_graph

pytestmark = pytest.mark.gpu

EST_RTOL = 1e-9


def _entry(native):
    fn = native.lib().rmcm_estimate_noalloc
    fn.argtypes = [C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    fn.restype = C.c_int32
    return fn


def _close(a, b):
    nz = b != 0
    if not np.array_equal(a[~nz], b[~nz]):
        return False
    rel = np.abs(a[nz] - b[nz]) / np.abs(b[nz])
    return rel.max(initial=0.0) <= EST_RTOL


class _DeviceChain:
    """A chain's CSR arrays copied into device memory owned by the caller
    (torch tensors), with the pointer arrays the entry point takes."""

    def __init__(self, torch, leaves):
        self.L = len(leaves)
        self.rows = np.array([m.shape[0] for m in leaves], np.int64)
        self.cols = np.array([m.shape[1] for m in leaves], np.int64)
        self.keep = []
        for m in leaves:
            rp, col, _ = m.download(values=False)
            col = col.copy() if col.size else np.zeros(1, np.int32)
            self.keep.append((torch.from_numpy(rp).cuda(), torch.from_numpy(col).cuda()))
        torch.cuda.synchronize()
        self.rp_ptrs = (C.c_void_p * self.L)(*[t[0].data_ptr() for t in self.keep])
        self.col_ptrs = (C.c_void_p * self.L)(*[t[1].data_ptr() for t in self.keep])

    def call(self, fn, stream=None):
        got = np.full(self.L * self.L, -1.0)
        rc = fn(self.L, self.rows.ctypes.data, self.cols.ctypes.data, C.cast(self.rp_ptrs, C.c_void_p),
                C.cast(self.col_ptrs, C.c_void_p), got.ctypes.data, stream)
        return rc, got.reshape(self.L, self.L)


def test_noalloc_estimates_match_the_allocating_entry_point(native, engine):
    torch = pytest.importorskip("torch")
    fn = _entry(native)
    fx = load_fixture("dblp_small")
    hg = native.HeteroGraph.from_synthetic(engine, make_graph(fx))
    checked = 0
    for rec in fx["paths"]:
        if rec["len"] < 2:
            continue
        leaves = hg.leaves(rec["metapath"])
        ref = engine.estimate(leaves)
        dc = _DeviceChain(torch, leaves)
        for _ in range(2):
            rc, got = dc.call(fn)
            assert rc == native.OK, rc
            assert _close(got, ref), rec["metapath"]
        checked += 1
    assert checked >= 5


def test_noalloc_allocates_nothing_and_honours_the_callers_stream(native, engine):
    torch = pytest.importorskip("torch")
    fn = _entry(native)
    fx = load_fixture("dblp_small")
    hg = native.HeteroGraph.from_synthetic(engine, make_graph(fx))
    mp = "1-3-0-1-2-4-0-0-1"
    leaves = hg.leaves(mp)
    ref = engine.estimate(leaves)
    dc = _DeviceChain(torch, leaves)
    side = torch.cuda.Stream()
    rc, _ = dc.call(fn)                       # warm-up: set-up and lazy module loading
    assert rc == native.OK
    rc, _ = dc.call(fn, C.c_void_p(side.cuda_stream))
    assert rc == native.OK
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    rc, got = dc.call(fn)
    assert rc == native.OK and _close(got, ref)
    rc, got_side = dc.call(fn, C.c_void_p(side.cuda_stream))
    assert rc == native.OK and _close(got_side, ref)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)


def _hub_graph(native_synth):
    """Three vertex types (60, 12,000, 400); vertex 0 of type 0 links to
    6,000 type-1 vertices, far past the 4,096-entry row the allocating
    estimator hands to a whole CTA; every other row is short."""
    rng = np.random.default_rng(21)
    n0, n1, n2 = 60, 12_000, 400
    src0 = [np.zeros(6000, np.int64)]
    dst0 = [rng.choice(n1, 6000, replace=False).astype(np.int64)]
    for u in range(1, n0):
        k = int(rng.integers(1, 30))
        src0.append(np.full(k, u, np.int64))
        dst0.append(rng.choice(n1, k, replace=False).astype(np.int64))
    src1 = np.repeat(np.arange(n1, dtype=np.int64), rng.integers(1, 4, n1))
    dst1 = rng.integers(0, n2, src1.size).astype(np.int64)
    src1, dst1 = native_synth.dedup_pairs_keep_order(src1, dst1, n2)
    g = native_synth.SyntheticHIN("hub_long_row", [n0, n1, n2])
    g.relations = [native_synth.Relation(0, 1, 0, 1, np.concatenate(src0), np.concatenate(dst0)),
                   native_synth.Relation(1, 2, 2, 3, src1, dst1)]
    return g


def test_noalloc_long_row_matches_the_allocating_path_and_the_oracle(native, engine, oracle_mod):
    torch = pytest.importorskip("torch")
    from resmcm_ari_gb300 import synth
    fn = _entry(native)
    g = _hub_graph(synth)
    hg = native.HeteroGraph.from_synthetic(engine, g)
    og = oracle_mod.OracleGraph.from_synthetic(g)
    for mp in ("0-0-1-2-2", "0-0-1-2-2-3-1", "0-0-1-2-2-3-1-1-0"):
        leaves = hg.leaves(mp)
        assert max(np.diff(leaves[0].download(values=False)[0])) > 4096
        ref = engine.estimate(leaves)
        orc = og.estimate(mp, threads=1)
        assert _close(ref, orc), mp
        dc = _DeviceChain(torch, leaves)
        for _ in range(2):
            rc, got = dc.call(fn)
            assert rc == native.OK, rc
            assert _close(got, ref) and _close(got, orc), mp


def test_noalloc_refuses_a_chain_beyond_its_fixed_scratch(native):
    fn = _entry(native)
    fake = (C.c_void_p * 2)(1, 1)     # never dereferenced: the size check refuses first
    out = np.zeros(4)
    for rows in ([50_000_000, 50_000_000], [1 << 61, 50_000_000], [5, (1 << 62) + 3]):
        r = np.array(rows, np.int64)
        cols = np.array([r[1], 10], np.int64)
        rc = fn(2, r.ctypes.data, cols.ctypes.data, C.cast(fake, C.c_void_p), C.cast(fake, C.c_void_p),
                out.ctypes.data, None)
        assert rc == native.EINVAL, rows
