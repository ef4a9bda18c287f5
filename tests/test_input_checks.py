"""The C-ABI's host-side input checks, without a GPU: malformed graphs and
generator parameters are rejected with LVG_EINVAL and a message naming the
call, before any device work; well-formed ones pass the checks (on a machine
without a GPU they then fail at the first CUDA call, with LVG_ECUDA)."""
import ctypes

import numpy as np
import pytest

from conftest import ROOT  # noqa: F401  (puts the package on sys.path)


@pytest.fixture(scope="module")
def L(lvg):
    import lvg_build

    lvg_build.build_cuda()
    lib = ctypes.CDLL(lvg.lib_path())
    lib.lvg_last_error.restype = ctypes.c_char_p
    lib.lvg_graph_create_planted_partition.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_double,
                                                      ctypes.c_double, ctypes.c_uint64, ctypes.c_void_p]
    lib.lvg_graph_create_rmat.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                          ctypes.c_double, ctypes.c_int, ctypes.c_uint64, ctypes.c_void_p]
    lib.lvg_graph_create.argtypes = [ctypes.c_size_t] + [ctypes.c_void_p] * 5
    lib.lvg_graph_create_from_edges.argtypes = [ctypes.c_size_t, ctypes.c_size_t] + [ctypes.c_void_p] * 4
    lib.lvg_graph_destroy.argtypes = [ctypes.c_void_p]
    return lib


def _outcome(lvg, L, rc, g):
    """(status, message); a graph that was made (on a GPU machine) is destroyed."""
    if rc == lvg.LVG_OK:
        L.lvg_graph_destroy(g)
        return rc, ""
    return rc, L.lvg_last_error().decode()


def _create(lvg, L, off, key, w, ex, span=None, null_keys=False):
    off = np.asarray(off, np.uint64)
    key = np.asarray(key, np.uint32)
    w = np.asarray(w, np.float32)
    ex = None if ex is None else np.asarray(ex, np.uint8)
    g = ctypes.c_void_p()
    rc = L.lvg_graph_create(len(off) - 1 if span is None else span, off.ctypes.data,
                            None if null_keys else key.ctypes.data, None if null_keys else w.ctypes.data,
                            None if ex is None else ex.ctypes.data, ctypes.byref(g))
    return _outcome(lvg, L, rc, g)


GOOD = ([0, 1, 2, 2], [1, 0], [1, 1], [1, 1, 1])  # vertices 0-1 joined, vertex 2 isolated


@pytest.mark.parametrize("case,args,msg", [
    ("offsets[0] not 0", ([1, 1, 2, 2], [1, 0], [1, 1], None), "offsets[0] != 0"),
    ("offsets decrease", ([0, 2, 1, 2], [1, 0], [1, 1], None), "offsets not monotone"),
    ("neighbour beyond the span", ([0, 1, 2, 2], [3, 0], [1, 1], None), "neighbour id >= span"),
    ("absent vertex with edges", ([0, 1, 2, 2], [1, 0], [1, 1], [1, 0, 1]), "absent vertex with edges"),
])
def test_malformed_graph_is_rejected(lvg, L, case, args, msg):
    rc, m = _create(lvg, L, *args)
    assert rc == lvg.LVG_EINVAL, case
    assert m == "lvg_graph_create: " + msg, (case, m)


def test_graph_create_argument_checks(lvg, L):
    assert _create(lvg, L, *GOOD, null_keys=True) == (lvg.LVG_EINVAL, "lvg_graph_create: null keys/weights")
    # span 0
    g = ctypes.c_void_p()
    off = np.zeros(1, np.uint64)
    rc = L.lvg_graph_create(0, off.ctypes.data, None, None, None, ctypes.byref(g))
    assert (rc, L.lvg_last_error().decode()) == (lvg.LVG_EINVAL, "lvg_graph_create: bad argument")
    # no edges at all needs no keys
    rc, _ = _create(lvg, L, [0, 0, 0], [], [], None, null_keys=True)
    assert rc != lvg.LVG_EINVAL


def test_well_formed_graph_passes_the_checks(lvg, L):
    rc, m = _create(lvg, L, *GOOD)
    assert rc in (lvg.LVG_OK, lvg.LVG_ECUDA), (rc, m)
    rc, m = _create(lvg, L, GOOD[0], GOOD[1], GOOD[2], None)
    assert rc in (lvg.LVG_OK, lvg.LVG_ECUDA), (rc, m)


def test_edge_list_ids_are_checked(lvg, L):
    src, dst = np.array([1, 2], np.uint32), np.array([2, 9], np.uint32)
    g = ctypes.c_void_p()
    rc = L.lvg_graph_create_from_edges(3, 2, src.ctypes.data, dst.ctypes.data, None, ctypes.byref(g))
    assert _outcome(lvg, L, rc, g) == (lvg.LVG_EINVAL, "lvg_graph_create_from_edges: id >= span")
    dst[1] = 1
    rc = L.lvg_graph_create_from_edges(3, 2, src.ctypes.data, dst.ctypes.data, None, ctypes.byref(g))
    assert _outcome(lvg, L, rc, g)[0] in (lvg.LVG_OK, lvg.LVG_ECUDA)


@pytest.mark.parametrize("n,block,deg,p_in", [(0, 8, 4.0, 0.5), (100, 0, 4.0, 0.5), (100, 8, float("nan"), 0.5),
                                              (100, 8, -1.0, 0.5), (100, 8, 4.0, 1.5), (100, 8, 4.0, -0.1)])
def test_planted_partition_parameters_are_checked(lvg, L, n, block, deg, p_in):
    g = ctypes.c_void_p()
    rc = L.lvg_graph_create_planted_partition(n, block, deg, p_in, 1, ctypes.byref(g))
    assert _outcome(lvg, L, rc, g) == (lvg.LVG_EINVAL, "lvg_graph_create_planted_partition: bad argument")


@pytest.mark.parametrize("scale,ef,a,b,c", [(0, 16, .57, .19, .19), (31, 16, .57, .19, .19),
                                            (10, -1, .57, .19, .19), (10, 16, .6, .3, .2), (10, 16, -.1, .5, .3)])
def test_rmat_parameters_are_checked(lvg, L, scale, ef, a, b, c):
    g = ctypes.c_void_p()
    rc = L.lvg_graph_create_rmat(scale, ef, a, b, c, 1, 1, ctypes.byref(g))
    assert _outcome(lvg, L, rc, g) == (lvg.LVG_EINVAL, "lvg_graph_create_rmat: bad argument")


def test_noalloc_modularity_refuses_before_any_launch(lvg, L):
    """lvg_modularity_noalloc takes device pointers it cannot inspect: a NULL
    keys or weights array, or a span above its fixed 2^20 cap, is refused on
    the host (every case here fails its checks, so nothing is launched on any
    machine)."""
    f = L.lvg_modularity_noalloc
    f.argtypes = [ctypes.c_size_t] + [ctypes.c_void_p] * 5 + [ctypes.c_double, ctypes.c_double, ctypes.c_void_p,
                                                              ctypes.c_void_p]
    dummy = ctypes.c_uint64(0)
    p = ctypes.addressof(dummy)  # a non-NULL pointer; never dereferenced by a refused call
    out = ctypes.c_double(0.0)
    for keys, weights in ((None, p), (p, None)):
        rc = f(16, p, keys, weights, None, p, 0.0, 1.0, ctypes.addressof(out), None)
        assert (rc, L.lvg_last_error().decode()) == (
            lvg.LVG_EINVAL, "lvg_modularity_noalloc: null argument or empty span")
    rc = f((1 << 20) + 1, p, p, p, None, p, 0.0, 1.0, ctypes.addressof(out), None)
    assert rc == lvg.LVG_EINVAL and "LVG_NOALLOC_MAX_SPAN" in L.lvg_last_error().decode()
