"""ctypes bindings for the CPU oracle (test infrastructure only).

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this package; it is the checker, never the measured or
shipped path.

* ``OracleGraph`` wraps ``oracle/_build/liboracle.so``: a plain C + OpenMP
  restatement of efficient/resmcm.cpp (loader, RES estimator, DP, order,
  Boolean Gustavson) plus a counting Gustavson for exact path counts.
* ``RefGraph`` wraps ``oracle/_ref/libref_resmcm.so``: the reference source
  itself, compiled in place by ``oracle/Makefile``, driven through its own
  classes.  It exists only where the reference checkout does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_LIB_PATH = os.path.join(HERE, "_ref", "libref_resmcm.so")
REF_CLI_PATH = os.path.join(HERE, "_ref", "resmcm")
REF_NAIVE_LIB_PATH = os.path.join(HERE, "_ref", "libref_naive.so")
# checkout of swordzlim/RESMCM_ARI used to build the reference harness; unset
# means the location oracle/Makefile names
DEFAULT_REF = os.environ.get("RESMCM_REF_DIR") or None

MODE_BOOL, MODE_COUNT = 0, 1
ORC_OK, ORC_EOVERFLOW = 0, 3

_i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")


class OrcTimes(C.Structure):
    _fields_ = [("es", C.c_double), ("dp", C.c_double), ("spgemm", C.c_double), ("total", C.c_double)]


def build(ref_dir: str | None = None, quiet: bool = True) -> None:
    """Build liboracle.so, and the reference harness when its checkout exists."""
    out = subprocess.DEVNULL if quiet else None
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True, stdout=out)
    ref = ref_dir or DEFAULT_REF
    cmd = ["make", "-s", "-C", HERE, "ref-if-present"] + ([f"REF={ref}"] if ref else [])
    subprocess.run(cmd, check=True, stdout=out)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.orc_graph_load_text.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, C.POINTER(C.c_void_p)]
        L.orc_graph_from_arrays.argtypes = [C.c_int64, _i32p, _i64p, _i32p, _i32p, C.POINTER(C.c_void_p)]
        L.orc_graph_free.argtypes = [C.c_void_p]
        for f in ("orc_graph_n", "orc_graph_m"):
            getattr(L, f).argtypes = [C.c_void_p]
            getattr(L, f).restype = C.c_int64
        L.orc_graph_max_vt.argtypes = [C.c_void_p]
        L.orc_graph_max_vt.restype = C.c_int32
        L.orc_graph_dim.argtypes = [C.c_void_p, C.c_int32]
        L.orc_graph_dim.restype = C.c_int64
        L.orc_graph_export.argtypes = [C.c_void_p, _i32p, _i64p, _i32p, _i32p]
        L.orc_metapath_parse.argtypes = [C.c_char_p, _i32p, _i32p, C.c_int32, C.POINTER(C.c_int32)]
        L.orc_leaf.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, _i64p, C.c_void_p]
        L.orc_estimate.argtypes = [C.c_void_p, _i32p, _i32p, C.c_int32, C.c_int32, _f64p, C.POINTER(C.c_double)]
        L.orc_dp.argtypes = [_f64p, C.c_int32, _f64p, _i32p]
        L.orc_order.argtypes = [_i32p, C.c_int32, _i32p]
        L.orc_chain.argtypes = [C.c_void_p, C.c_char_p, C.c_int32, C.c_int32, C.POINTER(C.c_void_p),
                                C.POINTER(OrcTimes)]
        L.orc_chain_with_order.argtypes = [C.c_void_p, C.c_char_p, _i32p, C.c_int32, C.c_int32,
                                           C.POINTER(C.c_void_p), C.POINTER(OrcTimes)]
        L.orc_result_rows.argtypes = [C.c_void_p]
        L.orc_result_rows.restype = C.c_int64
        L.orc_result_nnz.argtypes = [C.c_void_p]
        L.orc_result_nnz.restype = C.c_int64
        L.orc_result_export.argtypes = [C.c_void_p, _i64p, C.c_void_p, C.c_void_p]
        L.orc_result_digest.argtypes = [C.c_void_p, C.POINTER(C.c_uint64)]
        L.orc_result_free.argtypes = [C.c_void_p]
        _lib = L
    return _lib


def parse_metapath(s: str):
    """MetaPath(string) grammar → (vertex types, edge types); raises ValueError."""
    vts = np.zeros(65, np.int32)
    ets = np.zeros(64, np.int32)
    n = C.c_int32(0)
    rc = lib().orc_metapath_parse(s.encode(), vts, ets, 64, C.byref(n))
    if rc != ORC_OK:
        raise ValueError(f"the meta-path is incorrect: {s!r} (status {rc})")
    return vts[:n.value + 1].copy(), ets[:n.value].copy()


def dp(c: np.ndarray):
    """Chain-order DP over an estimate matrix → (m, s, pairs)."""
    c = np.ascontiguousarray(c, np.float64)
    L = c.shape[0]
    m = np.zeros((L, L), np.float64)
    s = np.zeros((L, L), np.int32)
    lib().orc_dp(c.reshape(-1), L, m.reshape(-1), s.reshape(-1))
    pairs = np.zeros(max(0, 2 * (L - 1)), np.int32)
    if L > 1:
        lib().orc_order(s.reshape(-1), L, pairs)
    return m, s, pairs.reshape(-1, 2)


class OracleResult:
    def __init__(self, rowptr, col, val, nnz, times, status, digest=None):
        self.rowptr, self.col, self.val = rowptr, col, val
        self.nnz, self.times, self.status = nnz, times, status
        self.digest = digest


class OracleGraph:
    """A typed graph held by the C oracle."""

    def __init__(self, handle):
        self._h = C.c_void_p(handle)

    @classmethod
    def from_text(cls, graph: str, vertex: str, edge: str) -> "OracleGraph":
        h = C.c_void_p()
        rc = lib().orc_graph_load_text(graph.encode(), vertex.encode(), edge.encode(), C.byref(h))
        if rc != ORC_OK:
            raise ValueError(f"oracle text load failed with status {rc}")
        return cls(h.value)

    @classmethod
    def from_arrays(cls, vtype, adj_ptr, adj_nbr, adj_et) -> "OracleGraph":
        h = C.c_void_p()
        vtype = np.ascontiguousarray(vtype, np.int32)
        rc = lib().orc_graph_from_arrays(vtype.size, vtype, np.ascontiguousarray(adj_ptr, np.int64),
                                         np.ascontiguousarray(adj_nbr, np.int32),
                                         np.ascontiguousarray(adj_et, np.int32), C.byref(h))
        if rc != ORC_OK:
            raise ValueError(f"oracle graph build failed with status {rc}")
        return cls(h.value)

    @classmethod
    def from_synthetic(cls, g) -> "OracleGraph":
        ptr, nbr, et = g.adjacency()
        return cls.from_arrays(g.vertex_types(), ptr, nbr, et)

    def close(self):
        if self._h:
            lib().orc_graph_free(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def n(self):
        return lib().orc_graph_n(self._h)

    @property
    def m(self):
        return lib().orc_graph_m(self._h)

    def dim(self, vt: int) -> int:
        return lib().orc_graph_dim(self._h, vt)

    def export(self):
        n, m = self.n, self.m
        vt = np.zeros(n, np.int32)
        ptr = np.zeros(n + 1, np.int64)
        nbr = np.zeros(max(m, 1), np.int32)
        et = np.zeros(max(m, 1), np.int32)
        lib().orc_graph_export(self._h, vt, ptr, nbr, et)
        return vt, ptr, nbr[:m], et[:m]

    def leaf(self, src: int, sink: int, et: int):
        """Leaf CSR (local ids, graph.txt order, repeats kept)."""
        rows = self.dim(src)
        rp = np.zeros(rows + 1, np.int64)
        lib().orc_leaf(self._h, src, sink, et, rp, None)
        col = np.zeros(max(int(rp[-1]), 1), np.int32)
        lib().orc_leaf(self._h, src, sink, et, rp, col.ctypes.data)
        return rp, col[:int(rp[-1])]

    def estimate(self, metapath: str, threads: int = 1):
        vts, ets = parse_metapath(metapath)
        L = ets.size
        c = np.zeros(L * L, np.float64)
        es = C.c_double(0)
        rc = lib().orc_estimate(self._h, vts, ets, L, threads, c, C.byref(es))
        if rc != ORC_OK:
            raise ValueError(f"oracle estimate failed with status {rc}")
        return c.reshape(L, L)

    def chain(self, metapath: str, mode: int = MODE_COUNT, threads: int = 1, pairs=None,
              export: bool = True, digest: bool = False) -> OracleResult:
        """One chain through the oracle's executor.  ``export`` copies the
        result out (local ids, rows sorted); ``digest`` computes its
        order-free digest instead (the library's rmcm_mat_digest function)."""
        h = C.c_void_p()
        t = OrcTimes()
        if pairs is None:
            rc = lib().orc_chain(self._h, metapath.encode(), mode, threads, C.byref(h), C.byref(t))
        else:
            p = np.ascontiguousarray(np.asarray(pairs).reshape(-1), np.int32)
            rc = lib().orc_chain_with_order(self._h, metapath.encode(), p, mode, threads, C.byref(h),
                                            C.byref(t))
        if rc not in (ORC_OK, ORC_EOVERFLOW):
            raise ValueError(f"oracle chain failed with status {rc}")
        dg = None
        try:
            nnz = lib().orc_result_nnz(h)
            rowptr = col = val = None
            if digest:
                d = C.c_uint64(0)
                lib().orc_result_digest(h, C.byref(d))
                dg = int(d.value)
            if export:
                rows = lib().orc_result_rows(h)
                rowptr = np.zeros(rows + 1, np.int64)
                col = np.zeros(max(nnz, 1), np.int32)
                val = np.zeros(max(nnz, 1), np.uint64)
                lib().orc_result_export(h, rowptr, col.ctypes.data,
                                        val.ctypes.data if mode == MODE_COUNT else None)
                col, val = col[:nnz], (val[:nnz] if mode == MODE_COUNT else None)
        finally:
            lib().orc_result_free(h)
        times = {"es": t.es, "dp": t.dp, "spgemm": t.spgemm, "total": t.total}
        return OracleResult(rowptr, col, val, nnz, times, rc, dg)


# --------------------------------------------------------------------------
# the reference itself, compiled in place (only where its checkout exists)
# --------------------------------------------------------------------------

_ref = None


def ref_available() -> bool:
    return os.path.exists(REF_LIB_PATH)


def ref_lib():
    global _ref
    if _ref is None:
        L = C.CDLL(REF_LIB_PATH)
        L.ref_load.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p]
        L.ref_load.restype = C.c_void_p
        L.ref_free.argtypes = [C.c_void_p]
        L.ref_free_buf.argtypes = [C.c_void_p]
        L.ref_estimate.argtypes = [C.c_void_p, C.c_char_p, C.c_int, _f64p, _i32p, _i32p,
                                   C.POINTER(C.c_int32), _f64p]
        L.ref_chain.argtypes = [C.c_void_p, C.c_char_p, C.c_int, C.POINTER(C.c_int64), _f64p,
                                C.POINTER(C.c_int64), C.POINTER(C.POINTER(C.c_int64)),
                                C.POINTER(C.POINTER(C.c_int32))]
        _ref = L
    return _ref


def ref_naive_order(dims_by_type, vts):
    """The reference naive.cpp DP over type dimensions → (split, m, pairs)."""
    L = C.CDLL(REF_NAIVE_LIB_PATH)
    L.ref_naive_order.argtypes = [_i32p, C.c_int32, _i32p, C.c_int32, _i32p, _f64p, _i32p]
    dims = np.ascontiguousarray(dims_by_type, np.int32)
    v = np.ascontiguousarray(vts, np.int32)
    n = v.size - 1
    split = np.zeros(n * n, np.int32)
    m = np.zeros(n * n, np.float64)
    pairs = np.zeros(max(2 * (n - 1), 1), np.int32)
    L.ref_naive_order(dims, dims.size, v, n, split, m, pairs)
    return split.reshape(n, n), m.reshape(n, n), pairs[:2 * (n - 1)].reshape(-1, 2)


class RefGraph:
    """The reference's HeteroGraph, loaded from the reference text files."""

    def __init__(self, graph: str, vertex: str, edge: str):
        self._h = ref_lib().ref_load(graph.encode(), vertex.encode(), edge.encode())

    def close(self):
        if self._h:
            ref_lib().ref_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def estimate(self, metapath: str, threads: int = 1):
        """Reference c_, m_, s_ and pair list (threads=1: deterministic sums)."""
        L = parse_metapath(metapath)[1].size
        c = np.zeros(L * L, np.float64)
        m = np.zeros(L * L, np.float64)
        s = np.zeros(L * L, np.int32)
        pairs = np.zeros(max(2 * (L - 1), 1), np.int32)
        n = C.c_int32(0)
        ref_lib().ref_estimate(self._h, metapath.encode(), threads, c, s, pairs, C.byref(n), m)
        return c.reshape(L, L), m.reshape(L, L), s.reshape(L, L), pairs[:2 * (L - 1)].reshape(-1, 2)

    def chain(self, metapath: str, threads: int = 1):
        """Reference SSP_dynamic → (rowptr, sorted cols, nnz, times)."""
        nnz = C.c_int64(0)
        rows = C.c_int64(0)
        t = np.zeros(4, np.float64)
        rp = C.POINTER(C.c_int64)()
        col = C.POINTER(C.c_int32)()
        ref_lib().ref_chain(self._h, metapath.encode(), threads, C.byref(nnz), t, C.byref(rows),
                            C.byref(rp), C.byref(col))
        nnz, rows = nnz.value, rows.value
        rowptr = np.ctypeslib.as_array(rp, shape=(rows + 1,)).copy()
        cols = (np.ctypeslib.as_array(col, shape=(nnz,)).copy() if nnz else np.zeros(0, np.int32))
        ref_lib().ref_free_buf(C.cast(rp, C.c_void_p))
        ref_lib().ref_free_buf(C.cast(col, C.c_void_p))
        times = dict(zip(("es", "dp", "spgemm", "total"), t.tolist()))
        return rowptr, cols, nnz, times
