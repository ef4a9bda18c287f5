"""Resident hub tables (lvg_tuning.hub_tables): every vertex above degree
8192 of a unit-weight graph keeps its neighbour counts per community with the
state, and the dynamic methods' first pass evaluates it from that table.

The counts are exact integers, so the gains are those of a fresh scan: in
deterministic mode the results with tables must equal the results without
them and the oracle's CPU replay, bit for bit — for a table built by the call,
taken from the prior state's cache, carried through a stream of batches (each
batch's edges added to the tables) and kept up to date by the moves.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

METHODS = {"nd": 1, "ds": 2, "df": 3}


@pytest.fixture(scope="module")
def base(cuda):
    # R-MAT scale 16, edge factor 48: ~40 vertices above degree 8192, unit weights
    x = cuda.rmat(16, 48, seed=77)
    X = cuda.Graph(x)
    r = cuda.louvain_static(X, cuda.LouvainOptions(deterministic=True))
    X.close()
    return x, r


def _same(a, b):
    for u, v in zip(a, b):
        assert np.array_equal(u, v)


def _graph_with_batch(cuda, x, seed):
    Y = cuda.Graph(x)
    hb = cuda.random_batch(x, 3000, seed=seed)
    db = cuda.DeviceBatch(Y, hb)
    Y.apply_batch(db)
    return Y, db


@pytest.mark.parametrize("method", ["nd", "ds", "df"])
def test_tables_equal_scans_deterministic(cuda, orc, base, method):
    x, r0 = base
    Y, db = _graph_with_batch(cuda, x, 5)
    o = cuda.LouvainOptions(deterministic=True)
    prior = cuda.State(Y)
    prior.set(r0.membership, r0.vertexWeight, r0.communityWeight)
    outs = []
    for tables in (0, 1, 1):  # scans; tables built; tables from the prior's cache
        cuda.set_tuning(Y, hub_tables=tables)
        out = cuda.State(Y)
        info = cuda.run_resident(Y, METHODS[method], db, prior, out, o)
        st = Y.stats()
        outs.append((out.get(), info, st))
    (a, ia, sa), (b, ib, sb), (c, ic, sc) = outs
    assert sa["hub_table_slots"] == 0
    if method == "nd":  # naive-dynamic scans its hubs whatever the tuning (every vertex moves)
        assert sb["hub_table_slots"] == 0 and sc["hub_table_slots"] == 0
    else:
        assert sb["hub_table_slots"] > 0 and sb["hub_tables_built"] == 1
        assert sc["hub_table_slots"] > 0 and sc["hub_tables_built"] == 0
    _same(a, b)
    _same(a, c)
    for i in (ib, ic):
        assert (i["iterations"], i["passes"], i["affectedVertices"]) == (ia["iterations"], ia["passes"],
                                                                        ia["affectedVertices"])
    # and the oracle's CPU replay of the same rule, on the updated graph and the tidied batch
    m, vt, ct, info = orc.louvain(Y.download(), METHODS[method], db.download(), r0.membership, r0.vertexWeight,
                                  r0.communityWeight, threads=4, sync=True, colors=o.effective_colors())
    assert np.array_equal(b[0], m)
    assert np.array_equal(b[1], vt)
    assert np.array_equal(b[2], ct)
    assert (ib["iterations"], ib["passes"], ib["affectedVertices"]) == (info["iterations"], info["passes"],
                                                                        info["affectedVertices"])


def test_tables_through_a_stream(cuda, base):
    """A state carried through batches in place: each batch applied to the
    graph, then DF from the state's last result. With tables the state's
    tables take each batch's edges (no rebuild after the first call); the
    results equal a graph that scans, step by step."""
    x, r0 = base
    o = cuda.LouvainOptions(deterministic=True)
    A, B = cuda.Graph(x), cuda.Graph(x)
    cuda.set_tuning(A, hub_tables=1)
    cuda.set_tuning(B, hub_tables=0)
    sa, sb = cuda.State(A), cuda.State(B)
    for s in (sa, sb):
        s.set(r0.membership, r0.vertexWeight, r0.communityWeight)
    g = x
    prev_passes = None
    for step in range(5):
        hb = cuda.random_batch(g, 2000, seed=100 + step)
        da, dbb = cuda.DeviceBatch(A, hb), cuda.DeviceBatch(B, hb)
        A.apply_batch(da)
        B.apply_batch(dbb)
        ia = cuda.run_resident(A, cuda.METHOD_FRONTIER, da, sa, sa, o)
        built = A.stats()["hub_tables_built"]
        ib = cuda.run_resident(B, cuda.METHOD_FRONTIER, dbb, sb, sb, o)
        _same(sa.get(), sb.get())
        assert (ia["iterations"], ia["passes"]) == (ib["iterations"], ib["passes"])
        if prev_passes == 1:
            assert built == 0, step  # the previous step's tables plus this batch's edges
        prev_passes = ia["passes"]
        g = A.download()


def test_tables_async_quality(cuda, orc, base):
    """Asynchronous mode: the same modularity as the scan path (within the
    asynchronous tolerance), with the hubs evaluated from their tables."""
    x, r0 = base
    qs = {}
    for tables in (0, 1):
        Y, db = _graph_with_batch(cuda, x, 9)
        cuda.set_tuning(Y, hub_tables=tables)
        prior, out = cuda.State(Y), cuda.State(Y)
        prior.set(r0.membership, r0.vertexWeight, r0.communityWeight)
        for _ in range(3):
            cuda.run_resident(Y, cuda.METHOD_FRONTIER, db, prior, out)
        if tables:
            assert Y.stats()["hub_table_slots"] > 0
        qs[tables] = Y.modularity(out.get()[0])
    assert abs(qs[1] - qs[0]) <= 0.005, qs


def test_static_run_invalidates_tables(cuda, base):
    """A static run into a state replaces its membership: the state's tables
    are rebuilt by the next dynamic run from it."""
    x, r0 = base
    Y, db = _graph_with_batch(cuda, x, 11)
    o = cuda.LouvainOptions(deterministic=True)
    st = cuda.State(Y)
    st.set(r0.membership, r0.vertexWeight, r0.communityWeight)
    cuda.run_resident(Y, cuda.METHOD_FRONTIER, db, st, st, o)
    cuda.run_resident(Y, cuda.METHOD_STATIC, None, None, st, o)
    out = cuda.State(Y)
    cuda.run_resident(Y, cuda.METHOD_FRONTIER, db, st, out, o)
    assert Y.stats()["hub_tables_built"] == 1
    cuda.set_tuning(Y, hub_tables=0)
    ref = cuda.State(Y)
    cuda.run_resident(Y, cuda.METHOD_FRONTIER, db, st, ref, o)
    _same(out.get(), ref.get())


def test_tables_with_fresh_result_states(cuda, base):
    """Every call into a new result state (allocated and freed call by call,
    so its buffers land at old or new addresses): the hubs are evaluated from
    the tables on every call, and the results stay those of the first."""
    x, r0 = base
    Y, db = _graph_with_batch(cuda, x, 13)
    o = cuda.LouvainOptions(deterministic=True)
    prior = cuda.State(Y)
    prior.set(r0.membership, r0.vertexWeight, r0.communityWeight)
    first = None
    keep = []
    for k in range(8):
        if k % 3 == 2:
            keep.append(cuda.State(Y))  # shifts the next allocations
        out = cuda.State(Y)
        cuda.run_resident(Y, cuda.METHOD_FRONTIER, db, prior, out, o)
        st = Y.stats()
        assert st["hub_table_slots"] > 0 and st["move_bin_vertices"][11] > 0, (k, st["hub_table_slots"])
        got = out.get()
        if first is None:
            first = got
        else:
            _same(first, got)
        out.close()


def _host_df(cuda, G, hb, prior, o):
    return cuda.louvain_dynamic_frontier(G, hb, prior[0], prior[1], prior[2], o)


def test_host_calls_reuse_tables(cuda, orc, base):
    """The host-array entry points (lvg_frontier …) cache the tables of two
    memberships: the last prior that needed a build and the last result. A
    call whose uploaded prior equals one of them exactly takes its tables (no
    build), any other prior gets tables built for it. Deterministic results
    equal a graph that scans and the oracle's replay on every call."""
    x, r0 = base
    o = cuda.LouvainOptions(deterministic=True)
    y_hb = cuda.random_batch(x, 3000, seed=21)
    A, B = cuda.Graph(x), cuda.Graph(x)
    A.apply_batch(y_hb)
    tb = B.apply_batch(y_hb)  # the tidied batch, as main.cxx hands it to the methods
    cuda.set_tuning(A, hub_tables=1)
    cuda.set_tuning(B, hub_tables=0)
    y = B.download()
    prior0 = (r0.membership, r0.vertexWeight, r0.communityWeight)
    m, vt, ct, info = orc.louvain(y, 3, tb, *prior0, threads=4, sync=True, colors=o.effective_colors())
    other = cuda.louvain_static(cuda.Graph(y), o)  # a second, different prior
    prior1 = (other.membership, other.vertexWeight, other.communityWeight)
    built = []
    for prior in (prior0, prior0, prior1, prior1, prior0):
        ra = _host_df(cuda, A, tb, prior, o)
        built.append(A.stats()["hub_tables_built"])
        assert A.stats()["hub_table_slots"] > 0
        rb = _host_df(cuda, B, tb, prior, o)
        _same((ra.membership, ra.vertexWeight, ra.communityWeight),
              (rb.membership, rb.vertexWeight, rb.communityWeight))
        assert (ra.iterations, ra.passes, ra.affectedVertices) == (rb.iterations, rb.passes, rb.affectedVertices)
        if prior is prior0:
            _same((ra.membership, ra.vertexWeight, ra.communityWeight), (m, vt, ct))
    # built for prior0, taken; built for prior1 (in place of prior0: the
    # other cache holds the last result), taken; built for prior0 again
    assert built == [1, 0, 1, 0, 1], built


def test_host_calls_through_a_stream(cuda, base):
    """main.cxx's loop through the host entry points: each batch applied to
    the graph (lvg_graph_apply_batch), then DF from the previous call's
    result. The result's tables were cached by that call and took the
    batch's edges when it was applied, so no call after the first builds
    tables while the runs end after one pass; results equal a scanning graph."""
    x, r0 = base
    o = cuda.LouvainOptions(deterministic=True)
    A, B = cuda.Graph(x), cuda.Graph(x)
    cuda.set_tuning(A, hub_tables=1)
    cuda.set_tuning(B, hub_tables=0)
    pa = pb = (r0.membership, r0.vertexWeight, r0.communityWeight)
    g = x
    prev_passes = None
    for step in range(5):
        hb = cuda.random_batch(g, 2000, seed=300 + step)
        ta, tb = A.apply_batch(hb), B.apply_batch(hb)
        ra = _host_df(cuda, A, ta, pa, o)
        built = A.stats()["hub_tables_built"]
        rb = _host_df(cuda, B, tb, pb, o)
        _same((ra.membership, ra.vertexWeight, ra.communityWeight),
              (rb.membership, rb.vertexWeight, rb.communityWeight))
        assert (ra.iterations, ra.passes) == (rb.iterations, rb.passes)
        if prev_passes == 1:
            assert built == 0, step
        prev_passes = ra.passes
        pa = (ra.membership, ra.vertexWeight, ra.communityWeight)
        pb = (rb.membership, rb.vertexWeight, rb.communityWeight)
        g = A.download()


def test_state_tables_belong_to_the_state(cuda, base):
    """A state's hub tables are filled by calls on its graph but owned by the
    state: counted in the state's device bytes (not the graph's) and released
    with the state, which may outlive its graph."""
    x, r0 = base
    Y, db = _graph_with_batch(cuda, x, 9)
    cuda.set_tuning(Y, hub_tables=1)
    prior, out = cuda.State(Y), cuda.State(Y)
    prior.set(r0.membership, r0.vertexWeight, r0.communityWeight)
    before = (prior.device_bytes(), out.device_bytes())
    cuda.run_resident(Y, cuda.METHOD_FRONTIER, db, prior, out, cuda.LouvainOptions(deterministic=True))
    assert Y.stats()["hub_tables_built"] == 1
    assert prior.device_bytes() > before[0] and out.device_bytes() > before[1]
    g_bytes = Y.device_bytes()
    out.close()  # its tables go with it; the graph's count is untouched
    assert Y.device_bytes() == g_bytes
    db.close()
    Y.close()
    prior.close()  # after its graph
