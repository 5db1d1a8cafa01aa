"""The estimator entry point that allocates nothing, through the C ABI.

rmcm_estimate_noalloc exists for callers that may not allocate device memory
when they need an estimate (a framework that owns all device memory in its
own pool, a serving loop that forbids allocation after start-up, code that
records a stream into a graph).  They hand over the chain as device CSR
arrays they own; the entry point keeps its temporaries in a fixed device
array built into the library.  This test gives it the same chains as the
allocating entry point, rmcm_estimate, twice in a row (the second call reuses
the array the first one left behind) and checks every estimate against the
allocating one within the estimator tolerance of the parity tests, 1e-9
relative.  It also checks that a chain too large for the fixed array is
refused.  The file is collected last so that a failure here cannot hide the
other tests' results.
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
        L = len(leaves)
        # the same chain in device memory owned by the caller
        rows = np.array([m.shape[0] for m in leaves], np.int64)
        cols = np.array([m.shape[1] for m in leaves], np.int64)
        keep = []
        for m in leaves:
            rp, col, _ = m.download(values=False)
            keep.append((torch.from_numpy(rp).cuda(), torch.from_numpy(col.copy() if col.size else
                                                                          np.zeros(1, np.int32)).cuda()))
        torch.cuda.synchronize()
        rp_ptrs = (C.c_void_p * L)(*[t[0].data_ptr() for t in keep])
        col_ptrs = (C.c_void_p * L)(*[t[1].data_ptr() for t in keep])
        for _ in range(2):
            got = np.full(L * L, -1.0)
            rc = fn(L, rows.ctypes.data, cols.ctypes.data, C.cast(rp_ptrs, C.c_void_p), C.cast(col_ptrs, C.c_void_p),
                    got.ctypes.data, None)
            assert rc == native.OK, rc
            assert _close(got.reshape(L, L), ref), rec["metapath"]
        checked += 1
    assert checked >= 5


def test_noalloc_refuses_a_chain_beyond_its_fixed_scratch(native):
    fn = _entry(native)
    rows = np.array([50_000_000, 50_000_000], np.int64)
    cols = np.array([50_000_000, 10], np.int64)
    fake = (C.c_void_p * 2)(1, 1)     # never dereferenced: the size check refuses first
    out = np.zeros(4)
    rc = fn(2, rows.ctypes.data, cols.ctypes.data, C.cast(fake, C.c_void_p), C.cast(fake, C.c_void_p),
            out.ctypes.data, None)
    assert rc == native.EINVAL
