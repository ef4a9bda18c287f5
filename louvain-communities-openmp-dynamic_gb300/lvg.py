"""Python bindings of louvain-gb300 (ctypes over the C-ABI).

Mirrors the reference's Louvain interface (inc/louvain.hxx):

* :class:`LouvainOptions` — ``LouvainOptions`` (inc/louvain.hxx:30-63), same
  fields and defaults, plus ``deterministic``;
* :class:`LouvainResult` — ``LouvainResult<K, double>`` (inc/louvain.hxx:78-145);
* :func:`louvain_static`, :func:`louvain_naive_dynamic`,
  :func:`louvain_dynamic_delta_screening`, :func:`louvain_dynamic_frontier` —
  ``louvainStaticOmp`` / ``louvainNaiveDynamicOmp`` /
  ``louvainDynamicDeltaScreeningOmp`` / ``louvainDynamicFrontierOmp``
  (inc/louvain.hxx:1285, 1349, 1542, 1674), on a :class:`Graph` in HBM.

Every call runs on the GPU through ``liblouvain_gb300.so``. There is no CPU
fallback: if the library or a GPU is missing the call raises.
Host graphs and batches come from :mod:`graphgen` helpers in this module
(``liblvg_graphgen.so``).
"""
from __future__ import annotations

import atexit
import ctypes as C
import os
import weakref
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBDIR = os.path.join(HERE, "lib")

LVG_OK = 0
LVG_EINVAL = -22
LVG_ENOMEM = -12
LVG_ETIMEOUT = -62
LVG_ECUDA = -1000

METHOD_STATIC, METHOD_NAIVE, METHOD_DELTA, METHOD_FRONTIER = 0, 1, 2, 3
METHOD_NAMES = {METHOD_STATIC: "static", METHOD_NAIVE: "naive-dynamic", METHOD_DELTA: "delta-screening",
                METHOD_FRONTIER: "dynamic-frontier"}

_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
_u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")


class LvgError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


# ----------------------------------------------------------------- C structs

class _Options(C.Structure):
    _fields_ = [("repeat", C.c_int), ("resolution", C.c_double), ("tolerance", C.c_double),
                ("aggregationTolerance", C.c_double), ("toleranceDrop", C.c_double),
                ("maxIterations", C.c_int), ("maxPasses", C.c_int), ("deterministic", C.c_int),
                ("colors", C.c_int)]


class _Result(C.Structure):
    _fields_ = [("span", C.c_size_t), ("membership", C.POINTER(C.c_uint32)),
                ("vertexWeight", C.POINTER(C.c_double)), ("communityWeight", C.POINTER(C.c_double)),
                ("iterations", C.c_int), ("passes", C.c_int), ("time", C.c_float), ("markingTime", C.c_float),
                ("initializationTime", C.c_float), ("firstPassTime", C.c_float), ("localMoveTime", C.c_float),
                ("aggregationTime", C.c_float), ("affectedVertices", C.c_size_t), ("owned", C.c_int)]


class _Batch(C.Structure):
    _fields_ = [("num_deletions", C.c_size_t), ("del_src", C.c_void_p), ("del_dst", C.c_void_p),
                ("del_w", C.c_void_p), ("num_insertions", C.c_size_t), ("ins_src", C.c_void_p),
                ("ins_dst", C.c_void_p), ("ins_w", C.c_void_p)]


class _BatchBuf(C.Structure):
    _fields_ = [("num_deletions", C.c_size_t), ("del_src", C.c_void_p), ("del_dst", C.c_void_p),
                ("del_w", C.c_void_p), ("num_insertions", C.c_size_t), ("ins_src", C.c_void_p),
                ("ins_dst", C.c_void_p), ("ins_w", C.c_void_p)]


class _ServerOptions(C.Structure):
    _fields_ = [("workers", C.c_int), ("hbm_budget", C.c_size_t), ("method", C.c_int), ("louvain", _Options),
                ("coalesce", C.c_size_t)]


class _RequestInfo(C.Structure):
    _fields_ = [("ticket", C.c_uint64), ("graph", C.c_int), ("status", C.c_int), ("queue_ms", C.c_double),
                ("apply_ms", C.c_double), ("run_ms", C.c_double), ("latency_ms", C.c_double),
                ("iterations", C.c_int), ("passes", C.c_int), ("affected", C.c_uint64),
                ("tidy_deletions", C.c_size_t), ("tidy_insertions", C.c_size_t), ("group", C.c_uint64),
                ("coalesced", C.c_int)]


class _ServerStats(C.Structure):
    _fields_ = [("completed", C.c_uint64), ("failed", C.c_uint64), ("updates", C.c_uint64), ("graphs", C.c_size_t),
                ("hbm_reserved", C.c_size_t), ("p50_ms", C.c_double), ("p99_ms", C.c_double),
                ("max_ms", C.c_double), ("mean_ms", C.c_double), ("wall_s", C.c_double),
                ("updates_per_s", C.c_double), ("requests_per_s", C.c_double), ("mean_queue_ms", C.c_double),
                ("mean_apply_ms", C.c_double), ("mean_run_ms", C.c_double)]


class _Tuning(C.Structure):
    _fields_ = [("frontier_colors", C.c_int), ("concurrent_bins", C.c_int), ("fused_small", C.c_int),
                ("hub_chunk", C.c_uint32), ("big_blocks_per_sm", C.c_int), ("frontier_max_fraction", C.c_double),
                ("hub_tables", C.c_int), ("bin_max_degree", C.c_uint32 * 12),
                ("level_graphs", C.c_int), ("small_regs", C.c_int)]

    def as_dict(self) -> dict:
        return {k: (list(v) if k == "bin_max_degree" else v)
                for k, v in ((k, getattr(self, k)) for k, _ in self._fields_)}


class _Stats(C.Structure):
    _fields_ = [("move_kernel_ms", C.c_double), ("move_launches", C.c_uint64), ("move_vertices", C.c_uint64),
                ("move_edges", C.c_uint64), ("moves", C.c_uint64), ("aggregate_kernel_ms", C.c_double),
                ("aggregate_edges", C.c_uint64), ("aggregate_launches", C.c_uint64),
                ("kernel_launches", C.c_uint64), ("move_bin_ms", C.c_double * 12),
                ("move_bin_vertices", C.c_uint64 * 12), ("move_bin_edges", C.c_uint64 * 12),
                ("call_upload_ms", C.c_double), ("call_run_ms", C.c_double), ("call_download_ms", C.c_double),
                ("move_bin_overflow", C.c_uint64 * 12), ("hub_chunk_overflow", C.c_uint64),
                ("hub_table_slots", C.c_uint64), ("hub_table_overflow", C.c_uint64),
                ("hub_tables_built", C.c_uint64), ("host_syncs", C.c_uint64), ("level_graphs", C.c_uint64)]


class _Csr(C.Structure):
    _fields_ = [("span", C.c_size_t), ("num_edges", C.c_size_t), ("offsets", C.POINTER(C.c_uint64)),
                ("keys", C.POINTER(C.c_uint32)), ("weights", C.POINTER(C.c_float)),
                ("exists", C.POINTER(C.c_uint8))]


class _GBatch(C.Structure):
    _fields_ = [("num_deletions", C.c_size_t), ("num_insertions", C.c_size_t),
                ("del_src", C.POINTER(C.c_uint32)), ("del_dst", C.POINTER(C.c_uint32)),
                ("del_w", C.POINTER(C.c_float)), ("ins_src", C.POINTER(C.c_uint32)),
                ("ins_dst", C.POINTER(C.c_uint32)), ("ins_w", C.POINTER(C.c_float))]


class _Edges(C.Structure):
    _fields_ = [("n", C.c_size_t), ("src", C.POINTER(C.c_uint32)), ("dst", C.POINTER(C.c_uint32)),
                ("w", C.POINTER(C.c_float))]


# ----------------------------------------------------------------- loading

_lib = None
_gen = None


def lib_path() -> str:
    return os.path.join(LIBDIR, "liblouvain_gb300.so")


def gen_path() -> str:
    return os.path.join(LIBDIR, "liblvg_graphgen.so")


# Handles still alive at interpreter exit are released by _close_all, in
# dependency order (servers, batches and states before their graphs), while
# the CUDA runtime is still up: handles kept in module globals would otherwise
# be destroyed in an arbitrary order during finalisation.
_LIVE = {k: weakref.WeakSet() for k in ("server", "batch", "state", "pinned", "graph")}


def _close_all() -> None:
    for kind in ("server", "batch", "state", "pinned", "graph"):
        for obj in list(_LIVE[kind]):
            try:
                obj.close()
            except Exception:
                pass


atexit.register(_close_all)


def load_library() -> C.CDLL:
    """Load liblouvain_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    p = lib_path()
    if not os.path.exists(p):
        raise LvgError(LVG_ECUDA, f"{p} is missing: build it first (lvg_build.py); there is no CPU fallback")
    L = C.CDLL(p)
    vp, sz, i32, f64 = C.c_void_p, C.c_size_t, C.c_int, C.c_double
    L.lvg_last_error.restype = C.c_char_p
    L.lvg_options_default.argtypes = [C.POINTER(_Options)]
    L.lvg_graph_create.argtypes = [sz, _u64p, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(vp)]
    L.lvg_graph_destroy.argtypes = [vp]
    for n in ("lvg_graph_span", "lvg_graph_order", "lvg_graph_size"):
        getattr(L, n).argtypes = [vp]
        getattr(L, n).restype = sz
    L.lvg_static.argtypes = [vp, C.POINTER(_Options), C.POINTER(_Result)]
    for n in ("lvg_naive_dynamic", "lvg_delta_screening", "lvg_frontier"):
        getattr(L, n).argtypes = [vp, C.POINTER(_Batch), _u32p, _f64p, _f64p, C.POINTER(_Options),
                                  C.POINTER(_Result)]
    L.lvg_result_free.argtypes = [C.POINTER(_Result)]
    L.lvg_modularity.argtypes = [vp, _u32p, f64, f64, C.POINTER(f64)]
    L.lvg_edge_weight.argtypes = [vp, C.POINTER(f64)]
    L.lvg_host_alloc.argtypes = [sz]
    L.lvg_host_alloc.restype = vp
    L.lvg_host_free.argtypes = [vp]
    L.lvg_set_profiling.argtypes = [vp, i32]
    L.lvg_tuning_default.argtypes = [C.POINTER(_Tuning)]
    L.lvg_tuning_default.restype = None
    L.lvg_graph_get_tuning.argtypes = [vp, C.POINTER(_Tuning)]
    L.lvg_graph_set_tuning.argtypes = [vp, C.POINTER(_Tuning)]
    L.lvg_autotune.argtypes = [vp, i32, vp, vp, C.POINTER(_Options), i32, C.POINTER(_Tuning),
                               C.POINTER(C.c_double)]
    L.lvg_set_device.argtypes = [i32]
    L.lvg_modularity_noalloc.argtypes = [sz, vp, vp, vp, vp, vp, f64, f64, vp, vp]
    L.lvg_get_stats.argtypes = [vp, C.POINTER(_Stats)]
    L.lvg_state_create.argtypes = [vp, C.POINTER(vp)]
    L.lvg_state_set.argtypes = [vp, _u32p, _f64p, _f64p]
    L.lvg_state_get.argtypes = [vp, vp, vp, vp]
    L.lvg_state_destroy.argtypes = [vp]
    L.lvg_device_batch_create.argtypes = [vp, C.POINTER(_Batch), C.POINTER(vp)]
    L.lvg_device_batch_destroy.argtypes = [vp]
    L.lvg_run_resident.argtypes = [vp, i32, vp, vp, vp, C.POINTER(_Options), C.POINTER(_Result)]
    L.lvg_affected_vertices.argtypes = [vp, i32, C.POINTER(_Batch), _u32p, _f64p, _f64p, C.POINTER(_Options),
                                        vp, vp, vp]
    L.lvg_aggregate.argtypes = [vp, _u32p, _u32p, C.POINTER(sz), _u64p, vp, vp]
    L.lvg_graph_apply_batch.argtypes = [vp, C.POINTER(_Batch), vp]
    L.lvg_graph_apply_device_batch.argtypes = [vp, vp]
    L.lvg_graph_download.argtypes = [vp, _u64p, vp, vp, vp]
    L.lvg_graph_create_planted_partition.argtypes = [C.c_uint32, C.c_uint32, f64, f64, C.c_uint64, C.POINTER(vp)]
    L.lvg_graph_create_rmat.argtypes = [i32, f64, f64, f64, f64, i32, C.c_uint64, C.POINTER(vp)]
    L.lvg_graph_create_from_edges.argtypes = [sz, sz, vp, vp, vp, C.POINTER(vp)]
    L.lvg_graph_clone.argtypes = [vp, C.POINTER(vp)]
    L.lvg_device_batch_generate.argtypes = [vp, sz, sz, C.c_uint32, C.c_uint32, C.c_float, C.c_uint64,
                                            C.POINTER(vp)]
    L.lvg_device_batch_size.argtypes = [vp, C.POINTER(sz), C.POINTER(sz)]
    L.lvg_device_batch_download.argtypes = [vp, vp]
    L.lvg_device_batch_set.argtypes = [vp, C.POINTER(_Batch)]
    L.lvg_graph_device_bytes.argtypes = [vp]
    L.lvg_graph_device_bytes.restype = sz
    L.lvg_state_device_bytes.argtypes = [vp]
    L.lvg_state_device_bytes.restype = sz
    L.lvg_device_batch_device_bytes.argtypes = [vp]
    L.lvg_device_batch_device_bytes.restype = sz
    L.lvg_graph_trim.argtypes = [vp, i32]
    L.lvg_server_options_default.argtypes = [C.POINTER(_ServerOptions)]
    L.lvg_graph_footprint.argtypes = [sz, sz]
    L.lvg_graph_footprint.restype = sz
    L.lvg_server_create.argtypes = [C.POINTER(_ServerOptions), C.POINTER(vp)]
    L.lvg_server_add_graph.argtypes = [vp, vp, i32, vp, vp, vp, C.POINTER(i32)]
    L.lvg_server_submit.argtypes = [vp, i32, C.POINTER(_Batch), C.POINTER(C.c_uint64)]
    L.lvg_server_wait.argtypes = [vp, C.c_uint64, C.POINTER(_RequestInfo)]
    L.lvg_server_set_coalesce.argtypes = [vp, sz]
    L.lvg_server_drain.argtypes = [vp]
    L.lvg_server_stats.argtypes = [vp, i32, C.POINTER(_ServerStats)]
    L.lvg_server_membership.argtypes = [vp, i32, vp, vp, vp]
    L.lvg_server_destroy.argtypes = [vp]
    L.lvg_static_many.argtypes = [C.POINTER(vp), sz, C.POINTER(_Options), i32, i32, C.POINTER(_Result)]
    L.lvg_graph_create_union.argtypes = [C.POINTER(vp), sz, C.POINTER(vp)]
    L.lvg_vertex_weights.argtypes = [vp, vp]
    L.lvg_community_weights.argtypes = [vp, vp, vp, vp]
    L.lvg_union_graphs.argtypes = [vp, C.POINTER(sz)]
    L.lvg_static_union.argtypes = [vp, C.POINTER(_Options), C.POINTER(_Result)]
    _lib = L
    return L


def load_graphgen() -> C.CDLL:
    global _gen
    if _gen is not None:
        return _gen
    p = gen_path()
    if not os.path.exists(p):
        raise LvgError(LVG_EINVAL, f"{p} is missing: build it first (lvg_build.py)")
    G = C.CDLL(p)
    G.lvgg_last_error.restype = C.c_char_p
    G.lvgg_planted_partition.argtypes = [C.c_uint32, C.c_uint32, C.c_double, C.c_double, C.c_uint64,
                                         C.POINTER(_Csr)]
    G.lvgg_rmat.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int, C.c_uint64,
                            C.POINTER(_Csr)]
    G.lvgg_random_batch.argtypes = [C.POINTER(_Csr), C.c_size_t, C.c_double, C.c_uint64, C.POINTER(_GBatch)]
    G.lvgg_apply_batch.argtypes = [C.POINTER(_Csr), C.POINTER(_GBatch), C.POINTER(_Csr)]
    G.lvgg_reference_batch.argtypes = [C.POINTER(_Csr), C.c_size_t, C.c_size_t, C.c_uint32, C.c_uint32, C.c_float,
                                       C.c_uint64, C.POINTER(_GBatch)]
    G.lvgg_csr_free.argtypes = [C.POINTER(_Csr)]
    G.lvgg_temporal_open.argtypes = [C.c_char_p, C.c_int, C.POINTER(C.c_void_p)]
    G.lvgg_temporal_read.argtypes = [C.c_void_p, C.c_size_t, C.c_int, C.POINTER(_Edges)]
    G.lvgg_temporal_close.argtypes = [C.c_void_p]
    G.lvgg_temporal_write.argtypes = [C.c_char_p, C.POINTER(_Edges)]
    G.lvgg_csr_from_edges.argtypes = [C.c_size_t, C.POINTER(_Edges), C.POINTER(_Csr)]
    G.lvgg_temporal_drift.argtypes = [C.c_uint32, C.c_uint32, C.c_double, C.c_size_t, C.c_double, C.c_size_t,
                                      C.c_double, C.c_uint64, C.POINTER(_Edges)]
    G.lvgg_edges_free.argtypes = [C.POINTER(_Edges)]
    G.lvgg_batch_free.argtypes = [C.POINTER(_GBatch)]
    _gen = G
    return G


def _check(rc: int) -> None:
    if rc != LVG_OK:
        raise LvgError(rc, load_library().lvg_last_error().decode(errors="replace"))


# ----------------------------------------------------------------- host data

@dataclass
class HostGraph:
    """A CSR graph in host memory (numpy). Row u = keys[offsets[u]:offsets[u+1]]."""
    offsets: np.ndarray  # uint64 [span+1]
    keys: np.ndarray     # uint32
    weights: np.ndarray  # float32
    exists: np.ndarray   # uint8 [span]

    @property
    def span(self) -> int:
        return len(self.offsets) - 1

    @property
    def num_edges(self) -> int:
        return int(self.offsets[-1])

    @property
    def order(self) -> int:
        return int(self.exists.sum())

    def _struct(self) -> _Csr:
        c = _Csr()
        c.span = self.span
        c.num_edges = self.num_edges
        c.offsets = self.offsets.ctypes.data_as(C.POINTER(C.c_uint64))
        c.keys = self.keys.ctypes.data_as(C.POINTER(C.c_uint32))
        c.weights = self.weights.ctypes.data_as(C.POINTER(C.c_float))
        c.exists = self.exists.ctypes.data_as(C.POINTER(C.c_uint8))
        return c

    def degrees(self) -> np.ndarray:
        return np.diff(self.offsets).astype(np.int64)


@dataclass
class HostBatch:
    """A tidy batch update: both directions, sorted by (src, dst)."""
    del_src: np.ndarray
    del_dst: np.ndarray
    del_w: np.ndarray
    ins_src: np.ndarray
    ins_dst: np.ndarray
    ins_w: np.ndarray

    @property
    def num_deletions(self) -> int:
        return len(self.del_src)

    @property
    def num_insertions(self) -> int:
        return len(self.ins_src)

    def _struct(self) -> _Batch:
        b = _Batch()
        b.num_deletions = self.num_deletions
        b.del_src = self.del_src.ctypes.data
        b.del_dst = self.del_dst.ctypes.data
        b.del_w = self.del_w.ctypes.data
        b.num_insertions = self.num_insertions
        b.ins_src = self.ins_src.ctypes.data
        b.ins_dst = self.ins_dst.ctypes.data
        b.ins_w = self.ins_w.ctypes.data
        return b

    def _gstruct(self) -> _GBatch:
        b = _GBatch()
        b.num_deletions = self.num_deletions
        b.num_insertions = self.num_insertions
        P32, PF = C.POINTER(C.c_uint32), C.POINTER(C.c_float)
        b.del_src = self.del_src.ctypes.data_as(P32)
        b.del_dst = self.del_dst.ctypes.data_as(P32)
        b.del_w = self.del_w.ctypes.data_as(PF)
        b.ins_src = self.ins_src.ctypes.data_as(P32)
        b.ins_dst = self.ins_dst.ctypes.data_as(P32)
        b.ins_w = self.ins_w.ctypes.data_as(PF)
        return b

    @staticmethod
    def empty() -> "HostBatch":
        z32, zf = np.zeros(0, np.uint32), np.zeros(0, np.float32)
        return HostBatch(z32, z32.copy(), zf, z32.copy(), z32.copy(), zf.copy())


def _take_csr(c: _Csr) -> HostGraph:
    G = load_graphgen()
    S, X = c.span, c.num_edges
    g = HostGraph(np.ctypeslib.as_array(c.offsets, (S + 1,)).copy(),
                  np.ctypeslib.as_array(c.keys, (max(X, 1),))[:X].copy(),
                  np.ctypeslib.as_array(c.weights, (max(X, 1),))[:X].copy(),
                  np.ctypeslib.as_array(c.exists, (S,)).copy())
    G.lvgg_csr_free(C.byref(c))
    return g


def _take_edges(G, e: _Edges):
    n = e.n
    out = (np.ctypeslib.as_array(e.src, (max(n, 1),))[:n].copy(),
           np.ctypeslib.as_array(e.dst, (max(n, 1),))[:n].copy(),
           np.ctypeslib.as_array(e.w, (max(n, 1),))[:n].copy())
    G.lvgg_edges_free(C.byref(e))
    return out


def _edges_struct(src, dst, w):
    src = np.ascontiguousarray(src, np.uint32)
    dst = np.ascontiguousarray(dst, np.uint32)
    w = np.ascontiguousarray(w, np.float32)
    e = _Edges(len(src), src.ctypes.data_as(C.POINTER(C.c_uint32)), dst.ctypes.data_as(C.POINTER(C.c_uint32)),
               w.ctypes.data_as(C.POINTER(C.c_float)))
    return e, (src, dst, w)


class TemporalReader:
    """A SNAP temporal file read in order (lvgg_temporal_open/read; inc/snap.hxx:41-140)."""

    def __init__(self, path: str, weighted: bool = False):
        self._G = load_graphgen()
        self.h = C.c_void_p()
        if self._G.lvgg_temporal_open(path.encode(), int(weighted), C.byref(self.h)) != 0:
            raise LvgError(LVG_EINVAL, self._G.lvgg_last_error().decode())

    def read(self, lines: int, symmetric: bool = True):
        """The next `lines` lines as (src, dst, w), both directions when symmetric."""
        e = _Edges()
        if self._G.lvgg_temporal_read(self.h, lines, int(symmetric), C.byref(e)) != 0:
            raise LvgError(LVG_EINVAL, self._G.lvgg_last_error().decode())
        return _take_edges(self._G, e)

    def close(self) -> None:
        if self.h:
            self._G.lvgg_temporal_close(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def write_temporal(path: str, src, dst, w=None) -> None:
    """Edges as a SNAP temporal file ("u v t" lines)."""
    G = load_graphgen()
    e, keep = _edges_struct(src, dst, np.ones(len(src), np.float32) if w is None else w)
    if G.lvgg_temporal_write(path.encode(), C.byref(e)) != 0:
        raise LvgError(LVG_EINVAL, G.lvgg_last_error().decode())


def csr_from_edges(rows: int, src, dst, w=None) -> HostGraph:
    """The graph readTemporalOmpW builds from an edge list (lvgg_csr_from_edges)."""
    G = load_graphgen()
    e, keep = _edges_struct(src, dst, np.ones(len(src), np.float32) if w is None else w)
    c = _Csr()
    if G.lvgg_csr_from_edges(rows, C.byref(e), C.byref(c)) != 0:
        raise LvgError(LVG_EINVAL, G.lvgg_last_error().decode())
    return _take_csr(c)


def temporal_drift(n: int, communities: int, edges: int, sigma: float = 1.0, p_in: float = 0.85,
                   drift_every: int | None = None, drift: float = 0.01, seed: int = 42):
    """Synthetic temporal stream with drifting communities (lvgg_temporal_drift): (src, dst, w)."""
    G = load_graphgen()
    e = _Edges()
    every = max(1, edges // 20) if drift_every is None else drift_every
    if G.lvgg_temporal_drift(n, communities, sigma, edges, p_in, every, drift, seed, C.byref(e)) != 0:
        raise LvgError(LVG_EINVAL, G.lvgg_last_error().decode())
    return _take_edges(G, e)


def experiment_path() -> str:
    """The experiment driver (louvain_gb300_experiment), built beside the libraries."""
    return os.path.join(LIBDIR, "louvain_gb300_experiment")


def planted_partition(n: int, block: int, avg_degree: float, p_in: float, seed: int) -> HostGraph:
    """Seeded planted-partition graph, ids 1..n (vertex 0 absent)."""
    G = load_graphgen()
    c = _Csr()
    if G.lvgg_planted_partition(n, block, avg_degree, p_in, seed, C.byref(c)) != 0:
        raise LvgError(LVG_EINVAL, G.lvgg_last_error().decode())
    return _take_csr(c)


def rmat(scale: int, edge_factor: float = 16, a: float = 0.57, b: float = 0.19, c: float = 0.19,
         seed: int = 42, permute: bool = True) -> HostGraph:
    """Seeded R-MAT graph, ids 1..2^scale (vertex 0 absent)."""
    G = load_graphgen()
    cs = _Csr()
    if G.lvgg_rmat(scale, edge_factor, a, b, c, int(permute), seed, C.byref(cs)) != 0:
        raise LvgError(LVG_EINVAL, G.lvgg_last_error().decode())
    return _take_csr(cs)


def _take_batch(G, gb) -> HostBatch:
    def arr(p, n, dt):
        return np.ctypeslib.as_array(p, (max(n, 1),))[:n].copy().astype(dt, copy=False)

    nd, ni = gb.num_deletions, gb.num_insertions
    b = HostBatch(arr(gb.del_src, nd, np.uint32), arr(gb.del_dst, nd, np.uint32), arr(gb.del_w, nd, np.float32),
                  arr(gb.ins_src, ni, np.uint32), arr(gb.ins_dst, ni, np.uint32), arr(gb.ins_w, ni, np.float32))
    G.lvgg_batch_free(C.byref(gb))
    return b


def random_batch(x: HostGraph, num_updates: int, insertion_fraction: float = 0.8, seed: int = 7) -> HostBatch:
    """Tidy random batch: insertions of absent uniform pairs, edge-uniform deletions."""
    G = load_graphgen()
    cs = x._struct()
    gb = _GBatch()
    if G.lvgg_random_batch(C.byref(cs), num_updates, insertion_fraction, seed, C.byref(gb)) != 0:
        raise LvgError(LVG_EINVAL, G.lvgg_last_error().decode())
    return _take_batch(G, gb)


def reference_batch(x: HostGraph, deletions: int, insertions: int, begin: int = 1, range_: int | None = None,
                    weight: float = 1.0, seed: int = 7) -> HostBatch:
    """Untidy batch drawn as the reference's generateEdgeDeletions/Insertions
    (lvgg_reference_batch); equals DeviceBatch.generate on the same graph."""
    G = load_graphgen()
    cs = x._struct()
    gb = _GBatch()
    r = x.span - begin if range_ is None else range_
    if G.lvgg_reference_batch(C.byref(cs), deletions, insertions, begin, r, weight, seed, C.byref(gb)) != 0:
        raise LvgError(LVG_EINVAL, G.lvgg_last_error().decode())
    return _take_batch(G, gb)


def apply_batch(x: HostGraph, b: HostBatch) -> HostGraph:
    """x with the batch applied (remove deletions, add insertions)."""
    G = load_graphgen()
    cs = x._struct()
    gb = b._gstruct()
    y = _Csr()
    if G.lvgg_apply_batch(C.byref(cs), C.byref(gb), C.byref(y)) != 0:
        raise LvgError(LVG_EINVAL, G.lvgg_last_error().decode())
    return _take_csr(y)


# ----------------------------------------------------------------- options / results

@dataclass
class LouvainOptions:
    """LouvainOptions (inc/louvain.hxx:30-63); defaults as its constructor (:60)."""
    repeat: int = 1
    resolution: float = 1.0
    tolerance: float = 1e-2
    aggregationTolerance: float = 1.0
    toleranceDrop: float = 10.0
    maxIterations: int = 20
    maxPasses: int = 10
    deterministic: bool = False
    colors: int = 0  # 0 = library default (8 asynchronous, 16 deterministic)

    def _struct(self) -> _Options:
        return _Options(self.repeat, self.resolution, self.tolerance, self.aggregationTolerance,
                        self.toleranceDrop, self.maxIterations, self.maxPasses, int(self.deterministic),
                        int(self.colors))

    def effective_colors(self) -> int:
        """Class count of the deterministic replay (deterministic mode's default is 16)."""
        k = self.colors if self.colors > 0 else (16 if self.deterministic else 8)
        return max(1, min(64, k))


@dataclass
class LouvainResult:
    """LouvainResult<uint32_t, double> (inc/louvain.hxx:78-145)."""
    membership: np.ndarray
    vertexWeight: np.ndarray
    communityWeight: np.ndarray
    iterations: int = 0
    passes: int = 0
    time: float = 0.0
    markingTime: float = 0.0
    initializationTime: float = 0.0
    firstPassTime: float = 0.0
    localMoveTime: float = 0.0
    aggregationTime: float = 0.0
    affectedVertices: int = 0
    stats: dict = field(default_factory=dict)


def _scalars(r: _Result) -> dict:
    return dict(iterations=r.iterations, passes=r.passes, time=r.time, markingTime=r.markingTime,
                initializationTime=r.initializationTime, firstPassTime=r.firstPassTime,
                localMoveTime=r.localMoveTime, aggregationTime=r.aggregationTime,
                affectedVertices=r.affectedVertices)


# ----------------------------------------------------------------- device objects

class Graph:
    """A graph resident in HBM (``lvg_graph``)."""

    def __init__(self, g: HostGraph | None):
        L = load_library()
        self._L = L
        self.h = C.c_void_p()
        _LIVE["graph"].add(self)
        if g is None:  # filled by a generator classmethod
            return
        w = g.weights if g.num_edges else np.zeros(1, np.float32)
        k = g.keys if g.num_edges else np.zeros(1, np.uint32)
        _check(L.lvg_graph_create(g.span, g.offsets, k.ctypes.data, w.ctypes.data, g.exists.ctypes.data,
                                  C.byref(self.h)))

    @classmethod
    def planted_partition(cls, n: int, block: int, avg_degree: float, p_in: float, seed: int) -> "Graph":
        """Generated in HBM (lvg_graph_create_planted_partition); equals planted_partition()."""
        G = cls(None)
        _check(G._L.lvg_graph_create_planted_partition(n, block, avg_degree, p_in, seed, C.byref(G.h)))
        return G

    @classmethod
    def rmat(cls, scale: int, edge_factor: float = 16, a: float = 0.57, b: float = 0.19, c: float = 0.19,
             permute: bool = True, seed: int = 42) -> "Graph":
        """Generated in HBM (lvg_graph_create_rmat); equals rmat()."""
        G = cls(None)
        _check(G._L.lvg_graph_create_rmat(scale, edge_factor, a, b, c, int(permute), seed, C.byref(G.h)))
        return G

    @classmethod
    def from_edges(cls, span: int, src, dst, w=None) -> "Graph":
        """Built in HBM from an edge list as readTemporalOmpW builds its graph
        (lvg_graph_create_from_edges); equals csr_from_edges(span - 1, ...)."""
        G = cls(None)
        src = np.ascontiguousarray(src, np.uint32)
        dst = np.ascontiguousarray(dst, np.uint32)
        wp = None if w is None else np.ascontiguousarray(w, np.float32)
        _check(G._L.lvg_graph_create_from_edges(span, len(src), src.ctypes.data, dst.ctypes.data,
                                                None if wp is None else wp.ctypes.data, C.byref(G.h)))
        return G

    def clone(self) -> "Graph":
        """A copy in HBM (lvg_graph_clone)."""
        G = Graph(None)
        _check(self._L.lvg_graph_clone(self.h, C.byref(G.h)))
        return G

    def vertex_weights(self) -> np.ndarray:
        """louvainVertexWeightsOmpW in FP64 (lvg_vertex_weights)."""
        out = np.zeros(self.span, np.float64)
        _check(self._L.lvg_vertex_weights(self.h, out.ctypes.data))
        return out

    def community_weights(self, membership, vtot=None) -> np.ndarray:
        """louvainCommunityWeightsOmpW in FP64 (lvg_community_weights); vtot None = the
        graph's vertex weights."""
        m = np.ascontiguousarray(membership, np.uint32)
        v = None if vtot is None else np.ascontiguousarray(vtot, np.float64)
        out = np.zeros(self.span, np.float64)
        _check(self._L.lvg_community_weights(self.h, m.ctypes.data, None if v is None else v.ctypes.data,
                                             out.ctypes.data))
        return out

    @classmethod
    def union(cls, graphs: "list[Graph]") -> "Graph":
        """The graphs' CSRs back to back in one graph in HBM (lvg_graph_create_union),
        for lvg_static_union; graph i's ids are shifted by the spans before it."""
        L = load_library()
        hs = (C.c_void_p * max(len(graphs), 1))(*[g.h for g in graphs])
        G = Graph(None)
        _check(L.lvg_graph_create_union(hs, len(graphs), C.byref(G.h)))
        G._union_spans = [g.span for g in graphs]
        return G

    @property
    def union_graphs(self) -> int:
        n = C.c_size_t()
        _check(self._L.lvg_union_graphs(self.h, C.byref(n)))
        return n.value

    def close(self) -> None:
        if self.h:
            self._L.lvg_graph_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def span(self) -> int:
        return int(self._L.lvg_graph_span(self.h))

    @property
    def order(self) -> int:
        return int(self._L.lvg_graph_order(self.h))

    @property
    def size(self) -> int:
        return int(self._L.lvg_graph_size(self.h))

    def edge_weight(self) -> float:
        out = C.c_double()
        _check(self._L.lvg_edge_weight(self.h, C.byref(out)))
        return out.value

    def modularity(self, membership: np.ndarray, M: float = 0.0, R: float = 1.0) -> float:
        out = C.c_double()
        _check(self._L.lvg_modularity(self.h, np.ascontiguousarray(membership, np.uint32), M, R, C.byref(out)))
        return out.value

    def set_profiling(self, on: bool) -> None:
        _check(self._L.lvg_set_profiling(self.h, int(on)))

    def device_bytes(self) -> int:
        """Device bytes held by the graph, its workspace and scratch (lvg_graph_device_bytes)."""
        return int(self._L.lvg_graph_device_bytes(self.h))

    def trim(self, level: int = 1) -> None:
        _check(self._L.lvg_graph_trim(self.h, level))

    def apply_batch(self, b: "HostBatch | DeviceBatch") -> "HostBatch | None":
        """Tidy a batch against the graph and apply it in place on the GPU (the
        reference's tidyBatchUpdateU + applyBatchUpdateOmpU). For a HostBatch
        returns the tidied batch (lvg_graph_apply_batch); a DeviceBatch is
        replaced by its tidied batch on the device (lvg_graph_apply_device_batch)."""
        if isinstance(b, DeviceBatch):
            _check(self._L.lvg_graph_apply_device_batch(self.h, b.h))
            return None
        s = b._struct()
        nd, ni = b.num_deletions, b.num_insertions
        t = HostBatch(np.zeros(max(nd, 1), np.uint32), np.zeros(max(nd, 1), np.uint32), np.zeros(max(nd, 1), np.float32),
                      np.zeros(max(ni, 1), np.uint32), np.zeros(max(ni, 1), np.uint32), np.zeros(max(ni, 1), np.float32))
        o = _BatchBuf(0, t.del_src.ctypes.data, t.del_dst.ctypes.data, t.del_w.ctypes.data,
                      0, t.ins_src.ctypes.data, t.ins_dst.ctypes.data, t.ins_w.ctypes.data)
        _check(self._L.lvg_graph_apply_batch(self.h, C.byref(s), C.byref(o)))
        kd, ki = o.num_deletions, o.num_insertions
        return HostBatch(t.del_src[:kd].copy(), t.del_dst[:kd].copy(), t.del_w[:kd].copy(),
                         t.ins_src[:ki].copy(), t.ins_dst[:ki].copy(), t.ins_w[:ki].copy())

    def download(self) -> HostGraph:
        """The graph as a compact host CSR (lvg_graph_download)."""
        S, X = self.span, self.size
        off = np.zeros(S + 1, np.uint64)
        key = np.zeros(max(X, 1), np.uint32)
        w = np.zeros(max(X, 1), np.float32)
        ex = np.zeros(S, np.uint8)
        _check(self._L.lvg_graph_download(self.h, off, key.ctypes.data, w.ctypes.data, ex.ctypes.data))
        return HostGraph(off, key[:X].copy(), w[:X].copy(), ex)

    def stats(self) -> dict:
        s = _Stats()
        _check(self._L.lvg_get_stats(self.h, C.byref(s)))
        out = {}
        for k, _ in _Stats._fields_:
            v = getattr(s, k)
            out[k] = list(v) if hasattr(v, "__len__") else v
        return out


def affected_vertices(y: Graph, method: int, batch: HostBatch, q, qvtot, qctot, o: LouvainOptions | None = None):
    """Initial affected flags of a method (lvg_affected_vertices). For delta-screening
    returns (vertices, neighbors, communities), else the flags array."""
    L = load_library()
    S = y.span
    f, nb, cm = np.zeros(S, np.uint8), np.zeros(S, np.uint8), np.zeros(S, np.uint8)
    b = (batch or HostBatch.empty())._struct()
    opt = (o or LouvainOptions())._struct()
    q, qvtot, qctot = _prior_arrays(S, q, qvtot, qctot)
    _check(L.lvg_affected_vertices(y.h, method, C.byref(b), q, qvtot, qctot,
                                   C.byref(opt), f.ctypes.data, nb.ctypes.data, cm.ctypes.data))
    return (f, nb, cm) if method == METHOD_DELTA else f


def aggregate(g: Graph, membership):
    """One aggregation step (lvg_aggregate): (renumbered membership, CN, offsets, keys, weights)."""
    L = load_library()
    S, X = g.span, g.size
    ren = np.zeros(S, np.uint32)
    cn = C.c_size_t()
    off = np.zeros(S + 1, np.uint64)
    keys = np.zeros(max(X, 1), np.uint32)
    w = np.zeros(max(X, 1), np.float64)
    _check(L.lvg_aggregate(g.h, np.ascontiguousarray(membership, np.uint32), ren, C.byref(cn), off,
                           keys.ctypes.data, w.ctypes.data))
    CN = cn.value
    E = int(off[CN])
    return ren, CN, off[:CN + 1].copy(), keys[:E].copy(), w[:E].copy()


def _prior_arrays(S: int, q, qvtot, qctot):
    """The prior state as the C types; the library reads span entries of each."""
    q = np.ascontiguousarray(q, np.uint32)
    qvtot = np.ascontiguousarray(qvtot, np.float64)
    qctot = np.ascontiguousarray(qctot, np.float64)
    if min(len(q), len(qvtot), len(qctot)) < S:
        raise LvgError(LVG_EINVAL, f"prior state: arrays shorter than the graph's span {S}")
    return q, qvtot, qctot


def _run(fn_name: str, g: Graph, batch: HostBatch | None, q, qvtot, qctot, o: LouvainOptions | None,
         out_buffers=None) -> LouvainResult:
    L = load_library()
    o = o or LouvainOptions()
    S = g.span
    r = _Result()
    keep = []
    if out_buffers is not None:
        m, vw, cw = out_buffers
        r.membership = m.ctypes.data_as(C.POINTER(C.c_uint32))
        r.vertexWeight = vw.ctypes.data_as(C.POINTER(C.c_double))
        r.communityWeight = cw.ctypes.data_as(C.POINTER(C.c_double))
    opt = o._struct()
    if fn_name == "lvg_static":
        _check(L.lvg_static(g.h, C.byref(opt), C.byref(r)))
    else:
        b = (batch or HostBatch.empty())._struct()
        keep.append(b)
        q, qvtot, qctot = _prior_arrays(S, q, qvtot, qctot)
        _check(getattr(L, fn_name)(g.h, C.byref(b), q, qvtot, qctot, C.byref(opt), C.byref(r)))
    if out_buffers is not None:
        m, vw, cw = out_buffers
    else:
        m = np.ctypeslib.as_array(r.membership, (S,)).copy()
        vw = np.ctypeslib.as_array(r.vertexWeight, (S,)).copy()
        cw = np.ctypeslib.as_array(r.communityWeight, (S,)).copy()
        L.lvg_result_free(C.byref(r))
    return LouvainResult(m, vw, cw, **_scalars(r), stats=g.stats())


def louvain_static(x: Graph, o: LouvainOptions | None = None, out_buffers=None) -> LouvainResult:
    """louvainStaticOmp (inc/louvain.hxx:1285) on the GPU."""
    return _run("lvg_static", x, None, None, None, None, o, out_buffers)


def louvain_naive_dynamic(y: Graph, batch: HostBatch, q, qvtot, qctot, o: LouvainOptions | None = None,
                          out_buffers=None) -> LouvainResult:
    """louvainNaiveDynamicOmp (inc/louvain.hxx:1349) on the GPU."""
    return _run("lvg_naive_dynamic", y, batch, q, qvtot, qctot, o, out_buffers)


def louvain_dynamic_delta_screening(y: Graph, batch: HostBatch, q, qvtot, qctot, o: LouvainOptions | None = None,
                                    out_buffers=None) -> LouvainResult:
    """louvainDynamicDeltaScreeningOmp (inc/louvain.hxx:1542) on the GPU."""
    return _run("lvg_delta_screening", y, batch, q, qvtot, qctot, o, out_buffers)


def louvain_dynamic_frontier(y: Graph, batch: HostBatch, q, qvtot, qctot, o: LouvainOptions | None = None,
                             out_buffers=None) -> LouvainResult:
    """louvainDynamicFrontierOmp (inc/louvain.hxx:1674) on the GPU."""
    return _run("lvg_frontier", y, batch, q, qvtot, qctot, o, out_buffers)


class State:
    """Membership / vertex weights / community weights resident in HBM (``lvg_state``)."""

    def __init__(self, g: Graph):
        self._L = load_library()
        self.g = g
        self.h = C.c_void_p()
        _LIVE["state"].add(self)
        _check(self._L.lvg_state_create(g.h, C.byref(self.h)))

    def set(self, q, qvtot, qctot) -> None:
        q, qvtot, qctot = _prior_arrays(self.g.span, q, qvtot, qctot)
        _check(self._L.lvg_state_set(self.h, q, qvtot, qctot))

    def get(self):
        S = self.g.span
        m = np.empty(S, np.uint32)
        vt = np.empty(S, np.float64)
        ct = np.empty(S, np.float64)
        _check(self._L.lvg_state_get(self.h, m.ctypes.data, vt.ctypes.data, ct.ctypes.data))
        return m, vt, ct

    def membership(self, out: np.ndarray | None = None) -> np.ndarray:
        m = out if out is not None else np.empty(self.g.span, np.uint32)
        _check(self._L.lvg_state_get(self.h, m.ctypes.data, None, None))
        return m

    def device_bytes(self) -> int:
        """Device bytes held by the state, its hub tables included (lvg_state_device_bytes)."""
        return int(self._L.lvg_state_device_bytes(self.h))

    def close(self) -> None:
        if self.h:
            self._L.lvg_state_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DeviceBatch:
    """A validated batch resident in HBM (``lvg_device_batch``)."""

    def __init__(self, g: Graph, b: HostBatch | None):
        self._L = load_library()
        self.g = g
        self.batch = b
        self.h = C.c_void_p()
        _LIVE["batch"].add(self)
        if b is None:  # filled by generate()
            return
        s = b._struct()
        _check(self._L.lvg_device_batch_create(g.h, C.byref(s), C.byref(self.h)))

    @classmethod
    def generate(cls, g: Graph, deletions: int, insertions: int, begin: int = 1, range_: int | None = None,
                 weight: float = 1.0, seed: int = 7) -> "DeviceBatch":
        """An untidy batch drawn in HBM as the reference's generators draw one
        (lvg_device_batch_generate); equals reference_batch() on the same graph."""
        d = cls(g, None)
        r = g.span - begin if range_ is None else range_
        _check(d._L.lvg_device_batch_generate(g.h, deletions, insertions, begin, r, weight, seed, C.byref(d.h)))
        return d

    def set(self, b: HostBatch) -> None:
        """Replace the contents with another host batch, reusing the device buffers (lvg_device_batch_set)."""
        s = b._struct()
        _check(self._L.lvg_device_batch_set(self.h, C.byref(s)))
        self.batch = b

    def size(self) -> tuple[int, int]:
        nd, ni = C.c_size_t(), C.c_size_t()
        _check(self._L.lvg_device_batch_size(self.h, C.byref(nd), C.byref(ni)))
        return nd.value, ni.value

    def download(self) -> HostBatch:
        nd, ni = self.size()
        t = HostBatch(np.zeros(max(nd, 1), np.uint32), np.zeros(max(nd, 1), np.uint32), np.zeros(max(nd, 1), np.float32),
                      np.zeros(max(ni, 1), np.uint32), np.zeros(max(ni, 1), np.uint32), np.zeros(max(ni, 1), np.float32))
        o = _BatchBuf(0, t.del_src.ctypes.data, t.del_dst.ctypes.data, t.del_w.ctypes.data,
                      0, t.ins_src.ctypes.data, t.ins_dst.ctypes.data, t.ins_w.ctypes.data)
        _check(self._L.lvg_device_batch_download(self.h, C.byref(o)))
        return HostBatch(t.del_src[:nd].copy(), t.del_dst[:nd].copy(), t.del_w[:nd].copy(),
                         t.ins_src[:ni].copy(), t.ins_dst[:ni].copy(), t.ins_w[:ni].copy())

    def close(self) -> None:
        if self.h:
            self._L.lvg_device_batch_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def run_resident(g: Graph, method: int, batch: DeviceBatch | None, prior: State | None, out: State,
                 o: LouvainOptions | None = None) -> dict:
    """lvg_run_resident: a method on HBM-resident inputs; returns the scalar result fields."""
    L = load_library()
    opt = (o or LouvainOptions())._struct()
    r = _Result()
    _check(L.lvg_run_resident(g.h, method, batch.h if batch else None, prior.h if prior else None, out.h,
                              C.byref(opt), C.byref(r)))
    return _scalars(r)


def tuning_default() -> dict:
    t = _Tuning()
    load_library().lvg_tuning_default(C.byref(t))
    return t.as_dict()


def get_tuning(g: Graph) -> dict:
    t = _Tuning()
    _check(load_library().lvg_graph_get_tuning(g.h, C.byref(t)))
    return t.as_dict()


def set_tuning(g: Graph, **knobs) -> dict:
    """Change some knobs of a graph's tuning (lvg_graph_set_tuning); returns the new tuning."""
    L = load_library()
    t = _Tuning()
    _check(L.lvg_graph_get_tuning(g.h, C.byref(t)))
    for k, v in knobs.items():
        if k == "bin_max_degree":  # a list of up to 12 limits (the rest 0)
            v = list(v) + [0] * (12 - len(v))
            v = (C.c_uint32 * 12)(*v)
        setattr(t, k, v)
    _check(L.lvg_graph_set_tuning(g.h, C.byref(t)))
    return t.as_dict()


def autotune(g: Graph, method: int, batch: "DeviceBatch | None" = None, prior: "State | None" = None,
             o: "LouvainOptions | None" = None, repeats: int = 3) -> "tuple[dict, float]":
    """lvg_autotune: the fastest launch-shape choices for this graph and workload, set on
    the graph; returns (tuning, ms)."""
    L = load_library()
    t = _Tuning()
    ms = C.c_double()
    opt = (o or LouvainOptions())._struct()
    _check(L.lvg_autotune(g.h, method, batch.h if batch else None, prior.h if prior else None, C.byref(opt),
                          repeats, C.byref(t), C.byref(ms)))
    return t.as_dict(), ms.value


def profiler_start() -> None:
    _check(load_library().lvg_profiler_start())


def profiler_stop() -> None:
    _check(load_library().lvg_profiler_stop())


def set_device(device: int) -> None:
    """Make `device` the current GPU of the calling thread (lvg_set_device)."""
    _check(load_library().lvg_set_device(device))


NOALLOC_MAX_SPAN = 1 << 20


def modularity_noalloc(span: int, d_offsets: int, d_keys: int, d_weights: int, d_exists: int | None,
                       d_membership: int, d_out: int, M: float = 0.0, R: float = 1.0, stream: int | None = None) -> None:
    """lvg_modularity_noalloc: modularity into *d_out from caller-owned device buffers
    (raw device addresses), without any device allocation; asynchronous on `stream`."""
    _check(load_library().lvg_modularity_noalloc(span, d_offsets, d_keys, d_weights, d_exists, d_membership,
                                                 M, R, d_out, stream))


class PinnedArray:
    """A numpy view of pinned host memory from lvg_host_alloc (for fast copies)."""

    def __init__(self, n: int, dtype):
        self._L = load_library()
        self.ptr = None
        _LIVE["pinned"].add(self)
        dt = np.dtype(dtype)
        self.ptr = self._L.lvg_host_alloc(max(1, n * dt.itemsize))
        if not self.ptr:
            raise LvgError(LVG_ENOMEM, "lvg_host_alloc failed")
        buf = (C.c_char * (n * dt.itemsize)).from_address(self.ptr)
        self.array = np.frombuffer(buf, dtype=dt, count=n)

    def close(self) -> None:
        if self.ptr:
            self.array = None
            self._L.lvg_host_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """A serving loop over graphs resident in HBM (``lvg_server``)."""

    def __init__(self, workers: int = 8, hbm_budget: int = 120 << 30, method: int = 3,
                 o: "LouvainOptions | None" = None, coalesce: int = 0):
        self._L = load_library()
        opt = _ServerOptions()
        self._L.lvg_server_options_default(C.byref(opt))
        opt.workers, opt.hbm_budget, opt.method, opt.coalesce = workers, hbm_budget, method, coalesce
        if o is not None:
            opt.louvain = o._struct()
        self.h = C.c_void_p()
        self.graphs: list[Graph] = []
        _LIVE["server"].add(self)
        _check(self._L.lvg_server_create(C.byref(opt), C.byref(self.h)))

    def add_graph(self, g: Graph, prior=None) -> int:
        """Make g resident (the server borrows it; keep g alive). prior = (q, qvtot, qctot) or None (static)."""
        gid = C.c_int()
        if prior is None:
            _check(self._L.lvg_server_add_graph(self.h, g.h, 0, None, None, None, C.byref(gid)))
        else:
            q, vt, ct = (np.ascontiguousarray(prior[0], np.uint32), np.ascontiguousarray(prior[1], np.float64),
                         np.ascontiguousarray(prior[2], np.float64))
            _check(self._L.lvg_server_add_graph(self.h, g.h, 0, q.ctypes.data, vt.ctypes.data, ct.ctypes.data,
                                                C.byref(gid)))
        self.graphs.append(g)
        return gid.value

    def submit(self, graph_id: int, b: HostBatch) -> int:
        t = C.c_uint64()
        s = b._struct()
        _check(self._L.lvg_server_submit(self.h, graph_id, C.byref(s), C.byref(t)))
        return t.value

    def wait(self, ticket: int) -> dict:
        r = _RequestInfo()
        rc = self._L.lvg_server_wait(self.h, ticket, C.byref(r))
        out = {k: getattr(r, k) for k, _ in _RequestInfo._fields_}
        if rc != LVG_OK:
            raise LvgError(rc, self._L.lvg_last_error().decode(errors="replace"))
        return out

    def drain(self) -> None:
        _check(self._L.lvg_server_drain(self.h))

    def set_coalesce(self, entries: int) -> None:
        """Coalescing cap for the groups formed from now on (0: one request per run)."""
        _check(self._L.lvg_server_set_coalesce(self.h, entries))

    def stats(self, reset: bool = False) -> dict:
        st = _ServerStats()
        _check(self._L.lvg_server_stats(self.h, int(reset), C.byref(st)))
        return {k: getattr(st, k) for k, _ in _ServerStats._fields_}

    def state(self, graph_id: int):
        S = self.graphs[graph_id].span
        m, vt, ct = np.empty(S, np.uint32), np.empty(S, np.float64), np.empty(S, np.float64)
        _check(self._L.lvg_server_membership(self.h, graph_id, m.ctypes.data, vt.ctypes.data, ct.ctypes.data))
        return m, vt, ct

    def close(self) -> None:
        if self.h:
            self._L.lvg_server_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def graph_footprint(span: int, edges: int) -> int:
    return int(load_library().lvg_graph_footprint(span, edges))


def louvain_static_union(u: Graph, o: "LouvainOptions | None" = None) -> "list[LouvainResult]":
    """Static Louvain on every graph of a union in one run (lvg_static_union):
    one LouvainResult per graph, as louvain_static gives it for the graph alone."""
    L = load_library()
    n = u.union_graphs
    res = (_Result * max(n, 1))()
    opt = (o or LouvainOptions())._struct()
    # every graph's result arrays are views into three arrays for the whole
    # union, passed as caller buffers: the library writes them in place
    spans = getattr(u, "_union_spans", None)
    if spans is None or len(spans) != n:
        raise RuntimeError("graph union without its graphs' spans (build it with Graph.union)")
    vb = np.concatenate([[0], np.cumsum(spans, dtype=np.int64)])
    allm = np.empty(int(vb[-1]) + 1, np.uint32)
    allv = np.empty(int(vb[-1]) + 1, np.float64)
    allc = np.empty(int(vb[-1]) + 1, np.float64)
    views = []
    for i in range(n):
        a, b = int(vb[i]), int(vb[i + 1])
        views.append((allm[a:b], allv[a:b], allc[a:b]))
        res[i].span = b - a
        res[i].membership = allm[a:].ctypes.data_as(C.POINTER(C.c_uint32))
        res[i].vertexWeight = allv[a:].ctypes.data_as(C.POINTER(C.c_double))
        res[i].communityWeight = allc[a:].ctypes.data_as(C.POINTER(C.c_double))
    _check(L.lvg_static_union(u.h, C.byref(opt), res))
    st = u.stats()
    return [LouvainResult(*views[i], **_scalars(res[i]), stats=st) for i in range(n)]


def louvain_static_many(graphs: "list[Graph]", o: "LouvainOptions | None" = None, workers: int = 16,
                        trim: int = 0) -> list[dict]:
    """Static Louvain on many graphs concurrently (lvg_static_many); per graph
    the scalar result fields and the membership."""
    L = load_library()
    n = len(graphs)
    hs = (C.c_void_p * max(n, 1))(*[g.h for g in graphs])
    res = (_Result * max(n, 1))()
    opt = (o or LouvainOptions())._struct()
    _check(L.lvg_static_many(hs, n, C.byref(opt), workers, trim, res))
    out = []
    for i, g in enumerate(graphs):
        r = res[i]
        d = _scalars(r)
        d["membership"] = np.ctypeslib.as_array(r.membership, (r.span,)).copy()
        L.lvg_result_free(C.byref(r))
        out.append(d)
    return out
