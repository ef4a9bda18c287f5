"""ctypes wrappers of the test oracle.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU legs of bench.py, as the checker or the timed CPU baseline; never by the
product path.

* :class:`Oracle` wraps ``_build/liblouvain_oracle.so``, the C restatement of
  the reference's Louvain hot path (oracle/louvain_oracle.c). It builds
  anywhere (gcc + OpenMP).
* :class:`Reference` wraps ``_ref/libref_louvain.so``, a harness compiled
  against the reference's own headers (oracle/ref_harness.cxx). It exists only
  where the reference checkout was available at build time.

Both take host graphs/batches as produced by the package's generators
(``HostGraph`` / ``HostBatch``: numpy arrays).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liblouvain_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libref_louvain.so")
STAGED_INC = os.path.join(HERE, "_ref", "src", "inc")

_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
_u32p = np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS")
_u64p = np.ctypeslib.ndpointer(np.uint64, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_vp = C.c_void_p
_sz = C.c_size_t


def build(ref: bool | None = None, ref_dir: str | None = None) -> None:
    """Compile the oracle and, where possible, the harness over the reference's headers.

    ref_dir: the reference checkout (default: $LVG_REFERENCE_DIR). With a
    checkout the harness is compiled from the headers where they lie, and the
    headers are also staged, unmodified, into the git-ignored _ref/src/ so that
    a machine without the checkout can build the harness itself. Without one,
    previously staged headers are used. ref=None builds the harness whenever
    either source exists; ref=True requires one; ref=False skips it.
    """
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    ref_dir = ref_dir or os.environ.get("LVG_REFERENCE_DIR")
    have_checkout = bool(ref_dir) and os.path.isdir(os.path.join(ref_dir, "inc"))
    have_staged = os.path.isfile(os.path.join(STAGED_INC, "main.hxx"))
    if ref is False:
        return
    if have_checkout:
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF_DIR={ref_dir}"], check=True)
        subprocess.run(["make", "-s", "-C", HERE, "stage", f"REF_DIR={ref_dir}"], check=True)
    elif have_staged:
        if _stale(REF_SO, [os.path.join(HERE, "ref_harness.cxx")]
                  + [os.path.join(STAGED_INC, f) for f in os.listdir(STAGED_INC)]):
            subprocess.run(["make", "-s", "-C", HERE, "ref-staged"], check=True)
    elif ref:
        raise FileNotFoundError("no reference checkout (LVG_REFERENCE_DIR) and no staged headers in " + STAGED_INC)


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def reference_available() -> bool:
    """Whether the harness over the reference's own headers is built and loads here."""
    if not os.path.exists(REF_SO):
        return False
    try:
        C.CDLL(REF_SO)
        return True
    except OSError:
        return False


class Options(C.Structure):
    _fields_ = [("repeat", C.c_int), ("resolution", C.c_double), ("tolerance", C.c_double),
                ("aggregationTolerance", C.c_double), ("toleranceDrop", C.c_double),
                ("maxIterations", C.c_int), ("maxPasses", C.c_int)]


def options(repeat=1, resolution=1.0, tolerance=1e-2, aggregationTolerance=1.0, toleranceDrop=10.0,
            maxIterations=20, maxPasses=10) -> Options:
    return Options(repeat, resolution, tolerance, aggregationTolerance, toleranceDrop, maxIterations, maxPasses)


class Info(C.Structure):
    _fields_ = [("iterations", C.c_int), ("passes", C.c_int), ("time", C.c_float), ("markingTime", C.c_float),
                ("initializationTime", C.c_float), ("firstPassTime", C.c_float), ("localMoveTime", C.c_float),
                ("aggregationTime", C.c_float), ("affectedVertices", C.c_uint64)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


def _batch_args(b):
    if b is None:
        z = np.zeros(1, np.uint32)
        zf = np.zeros(1, np.float32)
        return (0, z, z, zf, 0, z, z, zf)
    def nz(a, dt):
        a = np.ascontiguousarray(a, dt)
        return a if len(a) else np.zeros(1, dt)
    return (b.num_deletions, nz(b.del_src, np.uint32), nz(b.del_dst, np.uint32), nz(b.del_w, np.float32),
            b.num_insertions, nz(b.ins_src, np.uint32), nz(b.ins_dst, np.uint32), nz(b.ins_w, np.float32))


def _graph_args(g):
    k = g.keys if len(g.keys) else np.zeros(1, np.uint32)
    w = g.weights if len(g.weights) else np.zeros(1, np.float32)
    return (g.span, np.ascontiguousarray(g.offsets, np.uint64), np.ascontiguousarray(k, np.uint32),
            np.ascontiguousarray(w, np.float32), np.ascontiguousarray(g.exists, np.uint8))


class Oracle:
    """The C restatement (louvain_oracle.c)."""

    def __init__(self, path: str = ORACLE_SO):
        if not os.path.exists(path):
            build(ref=False)
        L = C.CDLL(path)
        G = [_sz, _u64p, _u32p, _f32p, _u8p]
        B = [_sz, _u32p, _u32p, _f32p, _sz, _u32p, _u32p, _f32p]
        L.orc_edge_weight.argtypes = G
        L.orc_edge_weight.restype = C.c_double
        L.orc_vertex_weights.argtypes = G + [_f64p]
        L.orc_update_weights.argtypes = B + [_u32p, _f64p, _f64p]
        L.orc_df_mark.argtypes = [_sz, _sz, _u32p, _u32p, _sz, _u32p, _u32p, _u32p, _u8p]
        L.orc_ds_mark.argtypes = G + [_sz, _u32p, _u32p, _sz, _u32p, _u32p, _f32p, _u32p, _f64p, _f64p,
                                      C.c_double, C.c_double, _u8p, _u8p, _u8p]
        L.orc_renumber.argtypes = [_sz, _u8p, _u32p]
        L.orc_renumber.restype = _sz
        L.orc_aggregate.argtypes = G + [_u32p, _u64p, _u32p, _u32p, _f64p]
        L.orc_aggregate.restype = _sz
        L.orc_modularity.argtypes = G + [_u32p, C.c_double, C.c_double]
        L.orc_modularity.restype = C.c_double
        run = G + [C.c_int] + B + [_u32p, _f64p, _f64p, C.POINTER(Options), C.c_int, _u32p, _f64p, _f64p,
                                   C.POINTER(Info)]
        szp = C.POINTER(C.c_size_t)
        L.orc_apply_batch.argtypes = G + B + [_u64p, _u32p, _f32p, _u8p, _u32p, _u32p, _f32p, szp, _u32p, _u32p,
                                              _f32p, szp]
        L.orc_apply_batch.restype = _sz
        L.orc_louvain.argtypes = run
        L.orc_louvain_sync.argtypes = run[:-4] + [C.c_int] + run[-4:]
        self.L = L

    def edge_weight(self, g) -> float:
        return self.L.orc_edge_weight(*_graph_args(g))

    def vertex_weights(self, g) -> np.ndarray:
        out = np.zeros(g.span, np.float64)
        self.L.orc_vertex_weights(*_graph_args(g), out)
        return out

    def update_weights(self, b, vcom, vtot, ctot):
        vt, ct = np.array(vtot, np.float64), np.array(ctot, np.float64)
        self.L.orc_update_weights(*_batch_args(b), np.ascontiguousarray(vcom, np.uint32), vt, ct)
        return vt, ct

    def df_mark(self, span, b, vcom) -> np.ndarray:
        f = np.zeros(span, np.uint8)
        a = _batch_args(b)
        self.L.orc_df_mark(span, a[0], a[1], a[2], a[4], a[5], a[6], np.ascontiguousarray(vcom, np.uint32), f)
        return f

    def ds_mark(self, g, b, vcom, vtot, ctot, M, R=1.0):
        S = g.span
        v, n, c = np.zeros(S, np.uint8), np.zeros(S, np.uint8), np.zeros(S, np.uint8)
        a = _batch_args(b)
        assert min(len(vcom), len(vtot), len(ctot)) >= S, "prior state shorter than the span"
        self.L.orc_ds_mark(*_graph_args(g), a[0], a[1], a[2], a[4], a[5], a[6], a[7],
                           np.ascontiguousarray(vcom, np.uint32), np.ascontiguousarray(vtot, np.float64),
                           np.ascontiguousarray(ctot, np.float64), M, R, v, n, c)
        return v, n, c

    def aggregate(self, g, vcom):
        """Renumber + aggregate; returns (renumbered vcom, CN, rows as dict c -> {d: w})."""
        S, X = g.span, g.num_edges
        vc = np.array(vcom, np.uint32)
        yoff = np.zeros(S + 1, np.uint64)
        ydeg = np.zeros(S + 1, np.uint32)
        yk = np.zeros(max(X, 1), np.uint32)
        yw = np.zeros(max(X, 1), np.float64)
        CN = self.L.orc_aggregate(*_graph_args(g), vc, yoff, ydeg, yk, yw)
        return vc, CN, _rows(CN, yoff, ydeg, yk, yw)

    def apply_batch(self, g, b):
        """tidyBatchUpdateU + applyBatchUpdateOmpU restated. Returns the graph as
        (offsets, keys, weights, exists) and the tidied batch as a tuple
        (ds, dd, dw, is, id, iw)."""
        S = g.span
        a = _batch_args(b)
        yoff = np.zeros(S + 1, np.uint64)
        cap = max(g.num_edges + a[4], 1)
        yk, yw, yex = np.zeros(cap, np.uint32), np.zeros(cap, np.float32), np.zeros(S, np.uint8)
        nd, ni = max(a[0], 1), max(a[4], 1)
        t = [np.zeros(nd, np.uint32), np.zeros(nd, np.uint32), np.zeros(nd, np.float32),
             np.zeros(ni, np.uint32), np.zeros(ni, np.uint32), np.zeros(ni, np.float32)]
        tnd, tni = C.c_size_t(), C.c_size_t()
        m = self.L.orc_apply_batch(*_graph_args(g), *a, yoff, yk, yw, yex, t[0], t[1], t[2], C.byref(tnd),
                                   t[3], t[4], t[5], C.byref(tni))
        tidy = tuple(x[:tnd.value].copy() for x in t[:3]) + tuple(x[:tni.value].copy() for x in t[3:])
        return (yoff, yk[:m].copy(), yw[:m].copy(), yex), tidy

    def modularity(self, g, membership, M=None, R=1.0) -> float:
        if M is None:
            M = self.edge_weight(g) / 2
        return self.L.orc_modularity(*_graph_args(g), np.ascontiguousarray(membership, np.uint32), M, R)

    def louvain(self, g, method=0, batch=None, q=None, qvtot=None, qctot=None, opts=None, threads=0, sync=False,
                colors=16):
        """Run a method. sync=True replays the GPU's deterministic mode with `colors` classes."""
        S = g.span
        q = np.zeros(S, np.uint32) if q is None else np.ascontiguousarray(q, np.uint32)
        qvtot = np.zeros(S, np.float64) if qvtot is None else np.ascontiguousarray(qvtot, np.float64)
        qctot = np.zeros(S, np.float64) if qctot is None else np.ascontiguousarray(qctot, np.float64)
        assert min(len(q), len(qvtot), len(qctot)) >= S, "prior state shorter than the span"
        m, vt, ct = np.zeros(S, np.uint32), np.zeros(S, np.float64), np.zeros(S, np.float64)
        info = Info()
        if sync:
            rc = self.L.orc_louvain_sync(*_graph_args(g), method, *_batch_args(batch), q, qvtot, qctot,
                                         C.byref(opts or options()), threads, colors, m, vt, ct, C.byref(info))
        else:
            rc = self.L.orc_louvain(*_graph_args(g), method, *_batch_args(batch), q, qvtot, qctot,
                                    C.byref(opts or options()), threads, m, vt, ct, C.byref(info))
        if rc != 0:
            raise RuntimeError(f"oracle louvain failed: {rc}")
        return m, vt, ct, info.as_dict()


def _rows(CN, yoff, ydeg, yk, yw):
    rows = []
    for c in range(CN):
        o, d = int(yoff[c]), int(ydeg[c])
        rows.append(dict(zip(yk[o:o + d].tolist(), yw[o:o + d].tolist())))
    return rows


class Reference:
    """Harness over the reference's own headers (ref_harness.cxx)."""

    def __init__(self, path: str = REF_SO):
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        L = C.CDLL(path)
        B = [_sz, _u32p, _u32p, _f32p, _sz, _u32p, _u32p, _f32p]
        L.ref_set_threads.argtypes = [C.c_int]
        L.ref_graph_new.argtypes = [_sz, _u64p, _u32p, _f32p, _u8p]
        L.ref_graph_new.restype = _vp
        L.ref_graph_free.argtypes = [_vp]
        L.ref_edge_weight.argtypes = [_vp]
        L.ref_edge_weight.restype = C.c_double
        L.ref_vertex_weights.argtypes = [_vp, _f64p]
        L.ref_update_weights.argtypes = [_vp] + B + [_u32p, _f64p, _f64p]
        L.ref_df_mark.argtypes = [_vp] + B + [_u32p, _u8p]
        L.ref_ds_mark.argtypes = [_vp] + B + [_u32p, _f64p, _f64p, C.c_double, C.c_double, _u8p, _u8p, _u8p]
        L.ref_aggregate.argtypes = [_vp, _u32p, _u64p, _u32p, _u32p, _f64p]
        L.ref_aggregate.restype = _sz
        szp = C.POINTER(C.c_size_t)
        L.ref_apply_batch.argtypes = [_vp] + B + [_u32p, _u32p, _f32p, szp, _u32p, _u32p, _f32p, szp]
        L.ref_graph_size.argtypes = [_vp]
        L.ref_graph_size.restype = _sz
        L.ref_graph_csr.argtypes = [_vp, _u64p, _u32p, _f32p, _u8p]
        L.ref_read_temporal.argtypes = [C.c_char_p, _sz, _sz]
        L.ref_read_temporal.restype = _vp
        L.ref_graph_csr.restype = _sz
        L.ref_modularity.argtypes = [_vp, _u32p, C.c_double, C.c_double]
        L.ref_modularity.restype = C.c_double
        L.ref_louvain.argtypes = [_vp, C.c_int] + B + [_u32p, _f64p, _f64p, C.c_int, C.c_double, C.c_double,
                                                       C.c_double, C.c_double, C.c_int, C.c_int, _u32p, _f64p,
                                                       _f64p, C.POINTER(Info)]
        self.L = L

    def threads(self, t: int) -> None:
        self.L.ref_set_threads(t)

    def read_temporal(self, path: str, rows: int, lines: int):
        """main.cxx's base graph: the first `lines` lines of a SNAP temporal file,
        read both ways and symmetrized; returns (offsets, keys, weights, exists)."""
        h = self.L.ref_read_temporal(path.encode(), rows, lines)
        try:
            S = rows + 1
            X = int(self.L.ref_graph_size(h))
            off = np.zeros(S + 1, np.uint64)
            k, w, ex = np.zeros(max(X, 1), np.uint32), np.zeros(max(X, 1), np.float32), np.zeros(S, np.uint8)
            m = self.L.ref_graph_csr(h, off, k, w, ex)
            return off, k[:m].copy(), w[:m].copy(), ex
        finally:
            self.L.ref_graph_free(h)

    def graph(self, g):
        S, off, k, w, ex = _graph_args(g)
        return _RefGraph(self, self.L.ref_graph_new(S, off, k, w, ex), g)


class _RefGraph:
    def __init__(self, ref: Reference, h, g):
        self.ref, self.h, self.g = ref, h, g

    def __del__(self):
        try:
            self.ref.L.ref_graph_free(self.h)
        except Exception:
            pass

    def edge_weight(self) -> float:
        return self.ref.L.ref_edge_weight(self.h)

    def vertex_weights(self) -> np.ndarray:
        out = np.zeros(self.g.span, np.float64)
        self.ref.L.ref_vertex_weights(self.h, out)
        return out

    def update_weights(self, b, vcom, vtot, ctot):
        vt, ct = np.array(vtot, np.float64), np.array(ctot, np.float64)
        self.ref.L.ref_update_weights(self.h, *_batch_args(b), np.ascontiguousarray(vcom, np.uint32), vt, ct)
        return vt, ct

    def df_mark(self, b, vcom) -> np.ndarray:
        f = np.zeros(self.g.span, np.uint8)
        self.ref.L.ref_df_mark(self.h, *_batch_args(b), np.ascontiguousarray(vcom, np.uint32), f)
        return f

    def ds_mark(self, b, vcom, vtot, ctot, M, R=1.0):
        S = self.g.span
        v, n, c = np.zeros(S, np.uint8), np.zeros(S, np.uint8), np.zeros(S, np.uint8)
        assert min(len(vcom), len(vtot), len(ctot)) >= S, "prior state shorter than the span"
        self.ref.L.ref_ds_mark(self.h, *_batch_args(b), np.ascontiguousarray(vcom, np.uint32),
                               np.ascontiguousarray(vtot, np.float64), np.ascontiguousarray(ctot, np.float64), M, R,
                               v, n, c)
        return v, n, c

    def aggregate(self, vcom):
        S, X = self.g.span, self.g.num_edges
        vc = np.array(vcom, np.uint32)
        yoff = np.zeros(S + 1, np.uint64)
        ydeg = np.zeros(S + 1, np.uint32)
        yk = np.zeros(max(X, 1), np.uint32)
        yw = np.zeros(max(X, 1), np.float64)
        CN = self.ref.L.ref_aggregate(self.h, vc, yoff, ydeg, yk, yw)
        return vc, CN, _rows(CN, yoff, ydeg, yk, yw)

    def apply_batch(self, b, csr: bool = True):
        """tidyBatchUpdateU + applyBatchUpdateOmpU on this graph, in place, as
        main.cxx runs them. Returns the graph as (offsets, keys, weights,
        exists) (None with csr=False) and the tidied batch as
        (ds, dd, dw, is, id, iw)."""
        a = _batch_args(b)
        nd, ni = max(a[0], 1), max(a[4], 1)
        t = [np.zeros(nd, np.uint32), np.zeros(nd, np.uint32), np.zeros(nd, np.float32),
             np.zeros(ni, np.uint32), np.zeros(ni, np.uint32), np.zeros(ni, np.float32)]
        tnd, tni = C.c_size_t(), C.c_size_t()
        self.ref.L.ref_apply_batch(self.h, *a, t[0], t[1], t[2], C.byref(tnd), t[3], t[4], t[5], C.byref(tni))
        tidy = tuple(x[:tnd.value].copy() for x in t[:3]) + tuple(x[:tni.value].copy() for x in t[3:])
        return (self.csr() if csr else None), tidy

    def size(self) -> int:
        return int(self.ref.L.ref_graph_size(self.h))

    def csr(self):
        S = self.g.span
        X = int(self.ref.L.ref_graph_size(self.h))
        yoff = np.zeros(S + 1, np.uint64)
        yk, yw, yex = np.zeros(max(X, 1), np.uint32), np.zeros(max(X, 1), np.float32), np.zeros(S, np.uint8)
        m = self.ref.L.ref_graph_csr(self.h, yoff, yk, yw, yex)
        return yoff, yk[:m].copy(), yw[:m].copy(), yex

    def modularity(self, membership, M=None, R=1.0) -> float:
        if M is None:
            M = self.edge_weight() / 2
        return self.ref.L.ref_modularity(self.h, np.ascontiguousarray(membership, np.uint32), M, R)

    def louvain(self, method=0, batch=None, q=None, qvtot=None, qctot=None, opts=None):
        """One call of the reference's entry point (opts.repeat repetitions
        inside it; info["time"] is their mean, the reference's own timer)."""
        S = self.g.span
        o = opts or options()
        q = np.zeros(S, np.uint32) if q is None else np.ascontiguousarray(q, np.uint32)
        qvtot = np.zeros(S, np.float64) if qvtot is None else np.ascontiguousarray(qvtot, np.float64)
        qctot = np.zeros(S, np.float64) if qctot is None else np.ascontiguousarray(qctot, np.float64)
        assert min(len(q), len(qvtot), len(qctot)) >= S, "prior state shorter than the span"
        m, vt, ct = np.zeros(S, np.uint32), np.zeros(S, np.float64), np.zeros(S, np.float64)
        info = Info()
        rc = self.ref.L.ref_louvain(self.h, method, *_batch_args(batch), q, qvtot, qctot, o.repeat, o.resolution,
                                    o.tolerance, o.aggregationTolerance, o.toleranceDrop, o.maxIterations,
                                    o.maxPasses, m, vt, ct, C.byref(info))
        if rc != 0:
            raise RuntimeError(f"reference louvain failed: {rc}")
        return m, vt, ct, info.as_dict()
