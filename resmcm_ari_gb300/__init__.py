"""GB300 (sm_103a) engine for RESMCM sparse matrix chain multiplication.

Python mirror of the reference program's interface (efficient/resmcm.cpp of
swordzlim/RESMCM_ARI) over the C ABI of ``libresmcm_gpu.so``
(``include/resmcm_gpu.h``):

==========================  ==============================================
reference                   here
==========================  ==============================================
``HeteroGraph(g, v, e)``    ``HeteroGraph.from_text(engine, g, v, e)``
``MetaPath(str)``           ``MetaPath(str)``  (same grammar, ``toString``)
``BoolMatrix(HIN, ...)``    ``HeteroGraph.leaf(src, sink, et)``
``getSparsities`` +         ``Engine.estimate(chain)``
``compute_sparsities``
DP + order                  ``Engine.order(c)``
``SpGEMM``                  ``Engine.spgemm(A, B)``
``SSP_dynamic``             ``Engine.chain(chain)`` / ``Engine.run_metapath``
``accuracy/res`` estimate   ``Engine.estimate_metapath``
==========================  ==============================================

Every product runs on the GPU through the native library; there is no CPU
fallback.  Importing the package never needs a GPU; creating an ``Engine``
does, and raises ``RuntimeError`` when the library or the device is missing.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_build", "libresmcm_gpu.so")
CLI_PATH = os.path.join(_PKG, "_build", "resmcm_gpu")
HEADER_PATH = os.path.join(os.path.dirname(_PKG), "include", "resmcm_gpu.h")

OK, EINVAL, ENOMEM, EOVERFLOW, ETIMEOUT, ECUDA, EIO, EPARSE, EINTERNAL = range(9)
ORDER_RES, ORDER_L2R, ORDER_DENSE = 0, 1, 2
VAL_U32, VAL_U64, VAL_AUTO = 0, 1, 2
_VAL_DTYPE = {VAL_U32: np.uint32, VAL_U64: np.uint64}


class RmcmError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{msg} (status {status})")
        self.status = status


class Opts(C.Structure):
    _fields_ = [("device", C.c_int32), ("valtype", C.c_int32), ("mem_budget_bytes", C.c_int64),
                ("stream", C.c_void_p)]


class Timings(C.Structure):
    _fields_ = [("total_s", C.c_double), ("spgemm_s", C.c_double), ("dp_s", C.c_double), ("es_s", C.c_double),
                ("nnz", C.c_int64), ("flops", C.c_int64), ("valtype", C.c_int32), ("n_products", C.c_int32)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


class Tuning(C.Structure):
    _fields_ = [("threads_per_row", C.c_int32), ("hash_max_flops", C.c_int32), ("dense_ratio", C.c_int32),
                ("warp_max_flops", C.c_int32), ("hash_load", C.c_double),
                ("gemm_inv_density", C.c_int32), ("gemm_min_mflops", C.c_int32)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


class ServerOpts(C.Structure):
    _fields_ = [("lanes", C.c_int32), ("reserved", C.c_int32), ("mem_budget_bytes", C.c_int64)]


class QueryResult(C.Structure):
    _fields_ = [("tag", C.c_int64), ("status", C.c_int32), ("graph", C.c_int32), ("nnz", C.c_int64),
                ("digest", C.c_uint64), ("t_submit", C.c_double), ("t_admit", C.c_double), ("t_done", C.c_double),
                ("est_bytes", C.c_double), ("es_s", C.c_double), ("dp_s", C.c_double), ("valtype", C.c_int32),
                ("lane", C.c_int32), ("error", C.c_char * 128)]

    def as_dict(self) -> dict:
        d = {f: getattr(self, f) for f, _ in self._fields_ if f != "error"}
        d["error"] = self.error.decode(errors="replace")
        return d


class ServerCounters(C.Structure):
    _fields_ = [("submitted", C.c_int64), ("completed", C.c_int64), ("rejected", C.c_int64),
                ("pending", C.c_int64), ("waiting", C.c_int64), ("running", C.c_int32), ("max_running", C.c_int32),
                ("lanes", C.c_int32), ("reserved_", C.c_int32), ("budget", C.c_int64), ("reserved", C.c_int64),
                ("peak_reserved", C.c_int64), ("kernel_launches", C.c_int64)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_ if f != "reserved_"}


class ProductStats(C.Structure):
    _fields_ = [("rows", C.c_int64), ("inner", C.c_int64), ("cols", C.c_int64),
                ("nnz_a", C.c_int64), ("nnz_b", C.c_int64), ("nnz_c", C.c_int64), ("flops", C.c_int64),
                ("touched_rows", C.c_int64), ("touched_nnz", C.c_int64),
                ("bytes_a", C.c_int64), ("bytes_b_touched", C.c_int64), ("bytes_c", C.c_int64),
                ("analyze_ms", C.c_double), ("symbolic_ms", C.c_double), ("numeric_ms", C.c_double),
                ("valtype", C.c_int32), ("bin_rows", C.c_int32 * 8),
                ("gemm_limbs", C.c_int32), ("gemm_inner", C.c_int64), ("gemm_ms", C.c_double)]

    def as_dict(self) -> dict:
        d = {f: getattr(self, f) for f, _ in self._fields_ if f != "bin_rows"}
        d["bin_rows"] = list(self.bin_rows)
        return d


_lib = None


def build(verbose: bool = False) -> str:
    from . import native_build
    return native_build.build(verbose=verbose)


def lib():
    """Load libresmcm_gpu.so (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"native library missing: {LIB_PATH} (run resmcm_ari_gb300.build())")
    L = C.CDLL(LIB_PATH)
    vp, i32, i64, f64p = C.c_void_p, C.c_int32, C.c_int64, C.POINTER(C.c_double)
    pp = C.POINTER(C.c_void_p)
    sig = {
        "rmcm_status_string": ([i32], C.c_char_p),
        "rmcm_create": ([pp, C.POINTER(Opts)], i32),
        "rmcm_destroy": ([vp], i32),
        "rmcm_last_error": ([vp], C.c_char_p),
        "rmcm_set_stream": ([vp, vp], i32),
        "rmcm_get_stream": ([vp], vp),
        "rmcm_mem_in_use": ([vp], i64),
        "rmcm_mem_peak": ([vp, i32], i64),
        "rmcm_kernel_launches": ([vp], i64),
        "rmcm_set_profiling": ([vp, i32], i32),
        "rmcm_get_product_stats": ([vp, C.POINTER(ProductStats), i32, C.POINTER(i32), i32], i32),
        "rmcm_graph_load_text": ([vp, C.c_char_p, C.c_char_p, C.c_char_p, pp], i32),
        "rmcm_graph_from_adjacency": ([vp, i64, vp, vp, vp, vp, pp], i32),
        "rmcm_graph_free": ([vp], i32),
        "rmcm_graph_info": ([vp, C.POINTER(i64), C.POINTER(i64), C.POINTER(i32)], i32),
        "rmcm_graph_dim": ([vp, i32], i64),
        "rmcm_metapath_parse": ([C.c_char_p, vp, vp, i32, C.POINTER(i32)], i32),
        "rmcm_metapath_format": ([vp, vp, i32, C.c_char_p, i64], i32),
        "rmcm_leaf": ([vp, vp, i32, i32, i32, i32, pp], i32),
        "rmcm_mat_upload": ([vp, i64, i64, vp, vp, vp, i32, pp], i32),
        "rmcm_mat_info": ([vp, C.POINTER(i64), C.POINTER(i64), C.POINTER(i64), C.POINTER(i32)], i32),
        "rmcm_mat_download": ([vp, vp, vp, vp, vp], i32),
        "rmcm_mat_free": ([vp, vp], i32),
        "rmcm_mat_download_async": ([vp, vp, vp, vp, vp], i32),
        "rmcm_transfers_wait": ([vp], i32),
        "rmcm_synchronize": ([vp], i32),
        "rmcm_estimate": ([vp, vp, i32, vp], i32),
        "rmcm_order": ([vp, vp, i32, vp, vp, vp], i32),
        "rmcm_spgemm": ([vp, vp, vp, pp], i32),
        "rmcm_chain": ([vp, vp, i32, vp, pp, C.POINTER(Timings)], i32),
        "rmcm_run_metapath": ([vp, vp, C.c_char_p, pp, C.POINTER(Timings)], i32),
        "rmcm_estimate_metapath": ([vp, vp, C.c_char_p, f64p], i32),
        "rmcm_set_order_mode": ([vp, i32], i32),
        "rmcm_order_l2r": ([i32, vp], i32),
        "rmcm_order_dense": ([vp, i32, vp, vp, vp], i32),
        "rmcm_graph_save": ([vp, C.c_char_p], i32),
        "rmcm_graph_load": ([vp, C.c_char_p, pp], i32),
        "rmcm_graph_global_ids": ([vp, i32, vp], i32),
        "rmcm_mat_save": ([vp, vp, C.c_char_p], i32),
        "rmcm_batch_create": ([vp, vp, vp, i32, i32, pp], i32),
        "rmcm_batch_create_fused": ([vp, vp, vp, i32, pp], i32),
        "rmcm_batch_run": ([vp, vp, vp, vp, f64p], i32),
        "rmcm_batch_info": ([vp, C.POINTER(i32), C.POINTER(i32), C.POINTER(i64), C.POINTER(i64)], i32),
        "rmcm_batch_free": ([vp, vp], i32),
        "rmcm_mat_digest": ([vp, vp, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)], i32),
        "rmcm_mat_digest_rows": ([vp, vp, i64, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)], i32),
        "rmcm_run_metapath_blocks": ([vp, vp, C.c_char_p, i64, BLOCK_FN, vp, C.POINTER(Timings)], i32),
        "rmcm_set_tuning": ([vp, C.POINTER(Tuning)], i32),
        "rmcm_get_tuning": ([vp, C.POINTER(Tuning)], i32),
        "rmcm_server_create": ([vp, C.POINTER(ServerOpts), pp], i32),
        "rmcm_server_add_graph": ([vp, vp, C.POINTER(i32)], i32),
        "rmcm_server_now": ([vp], C.c_double),
        "rmcm_server_submit": ([vp, i32, C.c_char_p, i64, C.c_double], i32),
        "rmcm_server_poll": ([vp, C.POINTER(QueryResult), i32, C.POINTER(i32), C.c_double], i32),
        "rmcm_server_drain": ([vp, C.c_double], i32),
        "rmcm_server_stats": ([vp, C.POINTER(ServerCounters)], i32),
        "rmcm_server_destroy": ([vp], i32),
    }
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _lib = L
    return L


# rmcm_block_fn: (user, row0, block) -> status
BLOCK_FN = C.CFUNCTYPE(C.c_int32, C.c_void_p, C.c_int64, C.c_void_p)


def order_l2r(length: int) -> np.ndarray:
    """Pair list of the left-to-right order (efficient/l2r.cpp:725-727)."""
    out = np.zeros(2 * (length - 1), np.int32)
    rc = lib().rmcm_order_l2r(length, _ptr(out))
    if rc != OK:
        raise RmcmError(rc, "order_l2r")
    return out.reshape(-1, 2)


def order_dense(dims_vt) -> tuple:
    """Dense-dimension DP of efficient/naive.cpp:506-523 → (split, cost, pairs)."""
    d = np.ascontiguousarray(dims_vt, np.int64)
    L = d.size - 1
    split = np.zeros(L * L, np.int32)
    cost = np.zeros(L * L, np.float64)
    pairs = np.zeros(max(2 * (L - 1), 1), np.int32)
    rc = lib().rmcm_order_dense(_ptr(d), L, _ptr(split), _ptr(cost), _ptr(pairs))
    if rc != OK:
        raise RmcmError(rc, "order_dense")
    return split.reshape(L, L), cost.reshape(L, L), pairs[:2 * (L - 1)].reshape(-1, 2)


def read_csr(path: str):
    """Read a result written by rmcm_mat_save → (rows, cols, rowptr, col, val)."""
    with open(path, "rb") as f:
        if f.read(8) != b"RMCMCSR1":
            raise ValueError(f"not a result file: {path}")
        rows, cols, nnz = np.frombuffer(f.read(24), np.int64)
        valtype = int(np.frombuffer(f.read(8), np.int32)[0])
        rp = np.frombuffer(f.read(8 * (rows + 1)), np.int64)
        col = np.frombuffer(f.read(4 * nnz), np.int32)
        val = np.frombuffer(f.read(_VAL_DTYPE[valtype]().itemsize * nnz), _VAL_DTYPE[valtype])
    return int(rows), int(cols), rp, col, val


def header_symbols() -> list:
    """Names of every entry point declared in include/resmcm_gpu.h."""
    import re
    text = open(HEADER_PATH).read()
    return re.findall(r"RMCM_API\s+[\w\s\*]+?\b(rmcm_\w+)\s*\(", text)


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


class MetaPath:
    """Meta-path string grammar of MetaPath(string), efficient/resmcm.cpp:269-299."""

    def __init__(self, s: str):
        vts = np.zeros(65, np.int32)
        ets = np.zeros(64, np.int32)
        n = C.c_int32(0)
        rc = lib().rmcm_metapath_parse(s.encode(), _ptr(vts), _ptr(ets), 64, C.byref(n))
        if rc != OK:
            raise ValueError(f"the meta-path is incorrect: {s!r}")
        self.vertex_types = vts[:n.value + 1].copy()
        self.edge_types = ets[:n.value].copy()
        self.path_len = n.value
        self.source = s

    def to_string(self) -> str:
        """MetaPath::toString, efficient/resmcm.cpp:301-308."""
        buf = C.create_string_buffer(16 * (2 * self.path_len + 1) + 16)
        lib().rmcm_metapath_format(_ptr(self.vertex_types), _ptr(self.edge_types), self.path_len, buf, len(buf))
        return buf.value.decode()

    toString = to_string


class Matrix:
    """A device-resident CSR owned by an Engine (or by a graph for leaves)."""

    def __init__(self, engine: "Engine", handle: int, owned: bool = True):
        self.engine = engine
        self._h = C.c_void_p(handle)
        self.owned = owned

    @property
    def shape(self):
        rows, cols, nnz, vt = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int32()
        lib().rmcm_mat_info(self._h, C.byref(rows), C.byref(cols), C.byref(nnz), C.byref(vt))
        return rows.value, cols.value

    @property
    def nnz(self) -> int:
        nnz = C.c_int64()
        lib().rmcm_mat_info(self._h, None, None, C.byref(nnz), None)
        return nnz.value

    @property
    def valtype(self) -> int:
        vt = C.c_int32()
        lib().rmcm_mat_info(self._h, None, None, None, C.byref(vt))
        return vt.value

    def download(self, values: bool = True):
        """(rowptr int64, col int32, val uint32/uint64 or None) on the host."""
        rows, _ = self.shape
        nnz = self.nnz
        rp = np.zeros(rows + 1, np.int64)
        col = np.zeros(max(nnz, 1), np.int32)
        val = np.zeros(max(nnz, 1), _VAL_DTYPE[self.valtype]) if values else None
        self.engine._check(lib().rmcm_mat_download(self.engine._h, self._h, _ptr(rp), _ptr(col),
                                                   _ptr(val) if values else None))
        return rp, col[:nnz], (val[:nnz] if values else None)

    def save(self, path: str):
        self.engine._check(lib().rmcm_mat_save(self.engine._h, self._h, path.encode()))

    def free(self):
        if self.owned and self._h:
            lib().rmcm_mat_free(self.engine._h, self._h)
        self._h = C.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class HeteroGraph:
    """Typed graph (HeteroGraph, efficient/resmcm.cpp:181-240) with a device leaf cache."""

    def __init__(self, engine: "Engine", handle: int):
        self.engine = engine
        self._h = C.c_void_p(handle)

    @classmethod
    def from_text(cls, engine: "Engine", graph: str, vertex: str, edge: str) -> "HeteroGraph":
        h = C.c_void_p()
        engine._check(lib().rmcm_graph_load_text(engine._h, graph.encode(), vertex.encode(), edge.encode(),
                                                 C.byref(h)))
        return cls(engine, h.value)

    @classmethod
    def from_adjacency(cls, engine: "Engine", vtype, adj_ptr, adj_nbr, adj_et) -> "HeteroGraph":
        vtype = np.ascontiguousarray(vtype, np.int32)
        adj_ptr = np.ascontiguousarray(adj_ptr, np.int64)
        adj_nbr = np.ascontiguousarray(adj_nbr, np.int32)
        adj_et = np.ascontiguousarray(adj_et, np.int32)
        h = C.c_void_p()
        engine._check(lib().rmcm_graph_from_adjacency(engine._h, vtype.size, _ptr(vtype), _ptr(adj_ptr),
                                                      _ptr(adj_nbr), _ptr(adj_et), C.byref(h)))
        return cls(engine, h.value)

    @classmethod
    def from_synthetic(cls, engine: "Engine", g) -> "HeteroGraph":
        ptr, nbr, et = g.adjacency()
        return cls.from_adjacency(engine, g.vertex_types(), ptr, nbr, et)

    @classmethod
    def load(cls, engine: "Engine", path: str) -> "HeteroGraph":
        """Binary graph cache written by save()."""
        h = C.c_void_p()
        engine._check(lib().rmcm_graph_load(engine._h, path.encode(), C.byref(h)))
        return cls(engine, h.value)

    def save(self, path: str):
        rc = lib().rmcm_graph_save(self._h, path.encode())
        if rc != OK:
            raise RmcmError(rc, f"cannot write graph cache {path}")

    def global_ids(self, vt: int) -> np.ndarray:
        out = np.zeros(max(self.dim(vt), 1), np.int32)
        lib().rmcm_graph_global_ids(self._h, vt, _ptr(out))
        return out[:self.dim(vt)]

    def info(self):
        n, m, mv = C.c_int64(), C.c_int64(), C.c_int32()
        lib().rmcm_graph_info(self._h, C.byref(n), C.byref(m), C.byref(mv))
        return n.value, m.value, mv.value

    def dim(self, vt: int) -> int:
        return lib().rmcm_graph_dim(self._h, vt)

    def leaf(self, src: int, sink: int, et: int, valtype: int = VAL_U32) -> Matrix:
        """BoolMatrix(HIN, vt, src, sink, et, n), efficient/resmcm.cpp:374-396 (graph-owned)."""
        h = C.c_void_p()
        self.engine._check(lib().rmcm_leaf(self.engine._h, self._h, src, sink, et, valtype, C.byref(h)))
        return Matrix(self.engine, h.value, owned=False)

    def leaves(self, metapath: str, valtype: int = VAL_U32) -> list:
        mp = MetaPath(metapath)
        return [self.leaf(int(mp.vertex_types[i]), int(mp.vertex_types[i + 1]), int(mp.edge_types[i]), valtype)
                for i in range(mp.path_len)]

    def close(self):
        if self._h:
            rc = lib().rmcm_graph_free(self._h)
            if rc != OK:
                raise RmcmError(rc, "graph_free: a batch still replays this graph's leaves")
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _mix64(x: np.ndarray) -> np.ndarray:
    """splitmix64 output function (Steele, Lea and Flood, OOPSLA 2014)."""
    x = x ^ (x >> np.uint64(30))
    x = x * np.uint64(0xBF58476D1CE4E5B9)
    x = x ^ (x >> np.uint64(27))
    x = x * np.uint64(0x94D049BB133111EB)
    return x ^ (x >> np.uint64(31))


def csr_digest(rowptr, col, val=None) -> tuple:
    """(nnz, digest) of a host CSR, the same function as rmcm_mat_digest:
    the sum mod 2^64 over entries (r, c, v) of mix(mix(r * 2^32 + c) + v)."""
    rowptr = np.asarray(rowptr, np.int64)
    col = np.asarray(col)
    nnz = int(rowptr[-1]) if rowptr.size else 0
    rows = np.repeat(np.arange(rowptr.size - 1, dtype=np.uint64), np.diff(rowptr))
    key = (rows << np.uint64(32)) | col[:nnz].astype(np.uint32).astype(np.uint64)
    v = np.ones(nnz, np.uint64) if val is None else np.asarray(val)[:nnz].astype(np.uint64)
    with np.errstate(over="ignore"):
        h = _mix64(_mix64(key) + v)
        return nnz, int(h.sum(dtype=np.uint64)) if nnz else 0


class Batch:
    """Meta-paths recorded once and replayed as one CUDA graph (rmcm_batch_*)."""

    def __init__(self, engine: "Engine", graph: "HeteroGraph", paths: list, lanes: int = 8, fused: bool = False):
        """fused: rmcm_batch_create_fused (estimator levels, DP and one
        block-diagonal SpGEMM per wave shared by every chain); else
        rmcm_batch_create (every chain's own launches over ``lanes`` streams)."""
        self.engine, self.graph, self.paths = engine, graph, list(paths)
        arr = (C.c_char_p * len(self.paths))(*[p.encode() for p in self.paths])
        h = C.c_void_p()
        if fused:
            engine._check(lib().rmcm_batch_create_fused(engine._h, graph._h, arr, len(self.paths), C.byref(h)))
        else:
            engine._check(lib().rmcm_batch_create(engine._h, graph._h, arr, len(self.paths), lanes, C.byref(h)))
        self._h = h

    def run(self):
        """Returns (nnz int64[count], digest uint64[count], device seconds)."""
        n = len(self.paths)
        nnz = np.zeros(n, np.int64)
        dig = np.zeros(n, np.uint64)
        sec = C.c_double()
        self.engine._check(lib().rmcm_batch_run(self.engine._h, self._h, _ptr(nnz), _ptr(dig), C.byref(sec)))
        return nnz, dig, sec.value

    def info(self) -> dict:
        c, ln, la, nd = C.c_int32(), C.c_int32(), C.c_int64(), C.c_int64()
        lib().rmcm_batch_info(self._h, C.byref(c), C.byref(ln), C.byref(la), C.byref(nd))
        return {"count": c.value, "lanes": ln.value, "launches_per_run": la.value, "graph_nodes": nd.value}

    def free(self):
        if getattr(self, "_h", None) and getattr(self.engine, "_h", None):
            lib().rmcm_batch_free(self.engine._h, self._h)
        self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class Server:
    """Query server over resident graphs (rmcm_server_*): admission by
    RES-predicted bytes, queries overlapping on ``lanes`` worker lanes."""

    def __init__(self, engine: "Engine", lanes: int = 8, mem_budget_bytes: int = 0):
        self.engine = engine
        self.graphs = []
        h = C.c_void_p()
        o = ServerOpts(lanes, 0, mem_budget_bytes)
        engine._check(lib().rmcm_server_create(engine._h, C.byref(o), C.byref(h)))
        self._h = h

    def add_graph(self, graph: "HeteroGraph") -> int:
        idx = C.c_int32()
        self.engine._check(lib().rmcm_server_add_graph(self._h, graph._h, C.byref(idx)))
        self.graphs.append(graph)
        return idx.value

    def now(self) -> float:
        return lib().rmcm_server_now(self._h)

    def submit(self, graph: int, metapath: str, tag: int, t_arrival: float = -1.0):
        self.engine._check(lib().rmcm_server_submit(self._h, graph, metapath.encode(), tag, t_arrival))

    def poll(self, wait_s: float = 0.0, cap: int = 1024) -> list:
        buf = (QueryResult * cap)()
        n = C.c_int32()
        self.engine._check(lib().rmcm_server_poll(self._h, buf, cap, C.byref(n), wait_s))
        return [buf[i].as_dict() for i in range(n.value)]

    def drain(self, timeout_s: float = 0.0):
        self.engine._check(lib().rmcm_server_drain(self._h, timeout_s))

    def stats(self) -> dict:
        st = ServerCounters()
        self.engine._check(lib().rmcm_server_stats(self._h, C.byref(st)))
        return st.as_dict()

    def close(self):
        if getattr(self, "_h", None):
            lib().rmcm_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Engine:
    """One handle on one GPU (rmcm_create); not thread-safe."""

    def __init__(self, device: int = 0, valtype: int = VAL_AUTO, mem_budget_bytes: int = 0, stream=None):
        o = Opts(device, valtype, mem_budget_bytes, stream)
        h = C.c_void_p()
        rc = lib().rmcm_create(C.byref(h), C.byref(o))
        if rc != OK:
            raise RmcmError(rc, f"rmcm_create failed: {lib().rmcm_status_string(rc).decode()}")
        self._h = h

    def _check(self, rc: int, allow=(OK,)):
        if rc not in allow:
            msg = lib().rmcm_last_error(self._h).decode() if self._h else ""
            raise RmcmError(rc, f"{lib().rmcm_status_string(rc).decode()}: {msg}")
        return rc

    def close(self):
        if getattr(self, "_h", None):
            lib().rmcm_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> int:
        return lib().rmcm_get_stream(self._h) or 0

    def set_stream(self, stream: int):
        self._check(lib().rmcm_set_stream(self._h, C.c_void_p(stream)))

    @property
    def mem_in_use(self) -> int:
        return lib().rmcm_mem_in_use(self._h)

    def mem_peak(self, reset: bool = False) -> int:
        """High-water mark of device bytes in use (rmcm_mem_peak)."""
        return lib().rmcm_mem_peak(self._h, 1 if reset else 0)

    @property
    def kernel_launches(self) -> int:
        return lib().rmcm_kernel_launches(self._h)

    def set_order_mode(self, mode: int):
        self._check(lib().rmcm_set_order_mode(self._h, mode))

    def set_profiling(self, level: int):
        self._check(lib().rmcm_set_profiling(self._h, level))

    def product_stats(self, reset: bool = True) -> list:
        n = C.c_int32()
        self._check(lib().rmcm_get_product_stats(self._h, None, 0, C.byref(n), 0))
        arr = (ProductStats * max(n.value, 1))()
        self._check(lib().rmcm_get_product_stats(self._h, arr, n.value, C.byref(n), 1 if reset else 0))
        return [arr[i].as_dict() for i in range(n.value)]

    def upload(self, rowptr, col, cols: int, val=None, valtype: int = VAL_U32) -> Matrix:
        rowptr = np.ascontiguousarray(rowptr, np.int64)
        col = np.ascontiguousarray(col, np.int32)
        v = None if val is None else np.ascontiguousarray(val, _VAL_DTYPE[valtype])
        h = C.c_void_p()
        self._check(lib().rmcm_mat_upload(self._h, rowptr.size - 1, cols, _ptr(rowptr), _ptr(col),
                                          None if v is None else _ptr(v), valtype, C.byref(h)))
        return Matrix(self, h.value)

    def upload_ptr(self, rowptr_ptr: int, col_ptr: int, rows: int, cols: int, val_ptr: int = 0,
                   valtype: int = VAL_U32) -> Matrix:
        """rmcm_mat_upload from raw host pointers (e.g. pinned buffers); val_ptr 0 = all ones."""
        h = C.c_void_p()
        self._check(lib().rmcm_mat_upload(self._h, rows, cols, C.c_void_p(rowptr_ptr), C.c_void_p(col_ptr),
                                          C.c_void_p(val_ptr) if val_ptr else None, valtype, C.byref(h)))
        return Matrix(self, h.value)

    @staticmethod
    def _chain_ptrs(chain):
        arr = (C.c_void_p * len(chain))(*[m._h.value for m in chain])
        return arr

    def estimate(self, chain) -> np.ndarray:
        L = len(chain)
        c = np.zeros(L * L, np.float64)
        self._check(lib().rmcm_estimate(self._h, self._chain_ptrs(chain), L, _ptr(c)))
        return c.reshape(L, L)

    def order(self, c: np.ndarray):
        c = np.ascontiguousarray(c, np.float64)
        L = c.shape[0]
        s = np.zeros(L * L, np.int32)
        m = np.zeros(L * L, np.float64)
        pairs = np.zeros(max(2 * (L - 1), 1), np.int32)
        self._check(lib().rmcm_order(self._h, _ptr(c), L, _ptr(s), _ptr(m), _ptr(pairs)))
        return s.reshape(L, L), m.reshape(L, L), pairs[:2 * (L - 1)].reshape(-1, 2)

    def spgemm(self, A: Matrix, B: Matrix) -> Matrix:
        h = C.c_void_p()
        self._check(lib().rmcm_spgemm(self._h, A._h, B._h, C.byref(h)), allow=(OK, EOVERFLOW))
        return Matrix(self, h.value)

    def chain(self, chain, pairs=None):
        h = C.c_void_p()
        t = Timings()
        p = None
        if pairs is not None:
            pa = np.ascontiguousarray(np.asarray(pairs).reshape(-1), np.int32)
            p = _ptr(pa)
        rc = self._check(lib().rmcm_chain(self._h, self._chain_ptrs(chain), len(chain), p, C.byref(h), C.byref(t)),
                         allow=(OK, EOVERFLOW))
        return Matrix(self, h.value), t.as_dict(), rc

    def run_metapath(self, graph: HeteroGraph, metapath: str, keep: bool = True):
        h = C.c_void_p()
        t = Timings()
        rc = self._check(lib().rmcm_run_metapath(self._h, graph._h, metapath.encode(),
                                                 C.byref(h) if keep else None, C.byref(t)),
                         allow=(OK, EOVERFLOW))
        return (Matrix(self, h.value) if keep else None), t.as_dict(), rc

    def run_metapath_blocks(self, graph: HeteroGraph, metapath: str, on_block, rows_per_block: int = 0):
        """rmcm_run_metapath_blocks: the result arrives in blocks of rows;
        on_block(row0, Matrix) is called for each (the matrix is valid only
        during the call).  Returns (timings, status)."""
        err = []

        def cb(_user, row0, blk):
            try:
                on_block(int(row0), Matrix(self, blk, owned=False))
                return OK
            except Exception as e:  # noqa: BLE001 -- re-raised after the call
                err.append(e)
                return EINVAL

        fn = BLOCK_FN(cb)
        t = Timings()
        rc = lib().rmcm_run_metapath_blocks(self._h, graph._h, metapath.encode(), int(rows_per_block), fn, None,
                                           C.byref(t))
        if err:
            raise err[0]
        self._check(rc, allow=(OK, EOVERFLOW))
        return t.as_dict(), rc

    def digest_rows(self, m: Matrix, row0: int) -> tuple:
        """(nnz, digest) of a block taken as rows row0.. of a larger matrix."""
        n, d = C.c_uint64(), C.c_uint64()
        self._check(lib().rmcm_mat_digest_rows(self._h, m._h, int(row0), C.byref(n), C.byref(d)))
        return n.value, d.value

    def get_tuning(self) -> dict:
        t = Tuning()
        self._check(lib().rmcm_get_tuning(self._h, C.byref(t)))
        return t.as_dict()

    def set_tuning(self, **kw):
        """Change some of threads_per_row, hash_max_flops, dense_ratio, warp_max_flops, hash_load,
        gemm_inv_density, gemm_min_mflops."""
        cur = self.get_tuning()
        bad = set(kw) - set(cur)
        if bad:
            raise ValueError(f"unknown tunables {sorted(bad)}")
        cur.update(kw)
        t = Tuning(int(cur["threads_per_row"]), int(cur["hash_max_flops"]), int(cur["dense_ratio"]),
                   int(cur["warp_max_flops"]), float(cur["hash_load"]), int(cur["gemm_inv_density"]),
                   int(cur["gemm_min_mflops"]))
        self._check(lib().rmcm_set_tuning(self._h, C.byref(t)))

    def batch(self, graph: HeteroGraph, paths: list, lanes: int = 8, fused: bool = False) -> Batch:
        return Batch(self, graph, paths, lanes, fused)

    def download_async(self, m: Matrix, rowptr_ptr: int, col_ptr: int, val_ptr: int = 0):
        """rmcm_mat_download_async into caller-owned (pinned) host buffers;
        they are valid after transfers_wait()."""
        self._check(lib().rmcm_mat_download_async(self._h, m._h, C.c_void_p(rowptr_ptr), C.c_void_p(col_ptr),
                                                  C.c_void_p(val_ptr or None)))

    def transfers_wait(self):
        self._check(lib().rmcm_transfers_wait(self._h))

    def synchronize(self):
        """rmcm_synchronize: all work of this handle is done."""
        self._check(lib().rmcm_synchronize(self._h))

    def digest(self, m: Matrix) -> tuple:
        """(nnz, digest) of a device matrix (rmcm_mat_digest)."""
        n, d = C.c_uint64(), C.c_uint64()
        self._check(lib().rmcm_mat_digest(self._h, m._h, C.byref(n), C.byref(d)))
        return n.value, d.value

    def estimate_metapath(self, graph: HeteroGraph, metapath: str) -> float:
        est = C.c_double()
        self._check(lib().rmcm_estimate_metapath(self._h, graph._h, metapath.encode(), C.byref(est)))
        return est.value
