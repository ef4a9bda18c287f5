"""Batch updates applied to the graph in HBM (lvg_graph_apply_batch /
lvg_graph_apply_device_batch) against the reference's host-side pair
tidyBatchUpdateU + applyBatchUpdateOmpU (inc/batch.hxx:202-209, 241-248), as
main.cxx:108-109 runs them before each dynamic call.

CPU: the oracle's restatement against the fixtures made by the reference's own
code (tests/golden/apply.npz: untidy batches, two in a row). GPU: the device
apply against the same fixtures and the oracle, bit-exact — graph rows, weights,
present flags, order, size, total weight and the tidied batch — through growth
into the overflow pool and a full re-layout, and the dynamic methods on the
device-updated graph against a graph uploaded from the same rows.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN

CASES = [("pp1k", 1), ("pp1k", 2), ("edge", 1), ("edge", 2)]


def _fixture():
    return np.load(os.path.join(GOLDEN, "apply.npz"))


def _graph(lvg, d, name, step):
    """The graph a step starts from: x for step 1, the previous result after."""
    if step == 1:
        p = f"{name}_x_"
        return lvg.HostGraph(d[p + "off"], d[p + "key"], d[p + "w"], d[p + "ex"])
    p = f"{name}_{step - 1}_y_"
    return lvg.HostGraph(d[p + "off"], d[p + "key"], d[p + "w"], d[p + "ex"])


def _batch(lvg, d, name, step):
    p = f"{name}_{step}_b_"
    return lvg.HostBatch(d[p + "ds"], d[p + "dd"], d[p + "dw"], d[p + "is"], d[p + "id"], d[p + "iw"])


def _expect(d, name, step):
    p = f"{name}_{step}_"
    y = tuple(d[p + "y_" + k] for k in ("off", "key", "w", "ex"))
    t = tuple(d[p + "t_" + k] for k in ("ds", "dd", "dw", "is", "id", "iw"))
    return y, t


def _tidy_tuple(b):
    return (b.del_src, b.del_dst, b.del_w, b.ins_src, b.ins_dst, b.ins_w)


def _same(a, b):
    return len(a) == len(b) and all(np.array_equal(np.asarray(x), np.asarray(y)) for x, y in zip(a, b))


# ------------------------------------------------------------------- CPU

@pytest.mark.parametrize("name,step", CASES)
def test_oracle_apply_matches_reference_fixture(lvg, orc, name, step):
    d = _fixture()
    x, b = _graph(lvg, d, name, step), _batch(lvg, d, name, step)
    y, t = orc.apply_batch(x, b)
    ey, et = _expect(d, name, step)
    assert _same(y, ey)
    assert _same(t, et)


def test_fixture_covers_the_untidy_cases(lvg):
    """The fixture batches hold what tidying removes, and the edge case makes
    absent vertices present."""
    d = _fixture()
    for name, step in CASES:
        b = _batch(lvg, d, name, step)
        _, t = _expect(d, name, step)
        assert len(t[0]) < b.num_deletions and len(t[3]) < b.num_insertions
    x = _graph(lvg, d, "edge", 1)
    ey, _ = _expect(d, "edge", 1)
    assert (ey[3].astype(int) - x.exists.astype(int)).max() == 1


def test_oracle_apply_of_a_tidy_batch_matches_the_generator(lvg, orc):
    x = lvg.planted_partition(2048, 128, 16, 0.8, 3)
    b = lvg.random_batch(x, 600, 0.8, seed=9)
    y, t = orc.apply_batch(x, b)
    g = lvg.apply_batch(x, b)
    assert _same(y, (g.offsets, g.keys, g.weights, g.exists))
    assert _same(t, _tidy_tuple(b))


# ------------------------------------------------------------------- GPU

def _download_matches(G, ey):
    h = G.download()
    assert np.array_equal(h.offsets, ey[0])
    assert np.array_equal(h.keys, ey[1])
    assert np.array_equal(h.weights, ey[2])
    assert np.array_equal(h.exists, ey[3])
    assert G.size == len(ey[1])
    assert G.order == int(ey[3].sum())


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["pp1k", "edge"])
def test_device_apply_matches_reference_two_batches_in_a_row(cuda, orc, name):
    d = _fixture()
    G = cuda.Graph(_graph(cuda, d, name, 1))
    for step in (1, 2):
        b = _batch(cuda, d, name, step)
        t = G.apply_batch(b)
        ey, et = _expect(d, name, step)
        _download_matches(G, ey)
        assert _same(_tidy_tuple(t), et)
        assert G.edge_weight() == orc.edge_weight(cuda.HostGraph(*ey))


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["pp1k", "edge"])
def test_device_batch_apply_tidies_the_batch_in_place(cuda, name):
    """A device batch applies once and then holds the tidied batch: a resident
    DF run from it equals lvg_frontier on the uploaded result with the tidied
    batch (deterministic mode: bit for bit)."""
    d = _fixture()
    x = _graph(cuda, d, name, 1)
    G = cuda.Graph(x)
    o = cuda.LouvainOptions(deterministic=True)
    r0 = cuda.louvain_static(G, o)
    prior = cuda.State(G)
    prior.set(r0.membership, r0.vertexWeight, r0.communityWeight)
    db = cuda.DeviceBatch(G, _batch(cuda, d, name, 1))
    G.apply_batch(db)
    ey, et = _expect(d, name, 1)
    _download_matches(G, ey)
    out = cuda.State(G)
    cuda.run_resident(G, cuda.METHOD_FRONTIER, db, prior, out, o)
    m, vt, ct = out.get()
    Y = cuda.Graph(cuda.HostGraph(*ey))
    tb = cuda.HostBatch(*et)
    r = cuda.louvain_dynamic_frontier(Y, tb, r0.membership, r0.vertexWeight, r0.communityWeight, o)
    assert np.array_equal(m, r.membership)
    assert np.array_equal(vt, r.vertexWeight) and np.array_equal(ct, r.communityWeight)
    with pytest.raises(cuda.LvgError) as e:
        G.apply_batch(db)
    assert e.value.code == cuda.LVG_EINVAL


@pytest.mark.gpu
def test_device_batch_reused_for_a_sequence(cuda):
    """One device batch refilled with lvg_device_batch_set for each step gives
    the same graph as a fresh device batch per step."""
    d = _fixture()
    A = cuda.Graph(_graph(cuda, d, "pp1k", 1))
    B = cuda.Graph(_graph(cuda, d, "pp1k", 1))
    db = None
    for step in (1, 2):
        b = _batch(cuda, d, "pp1k", step)
        if db is None:
            db = cuda.DeviceBatch(A, b)
        else:
            db.set(b)
        A.apply_batch(db)
        B.apply_batch(cuda.DeviceBatch(B, b))
        ha, hb = A.download(), B.download()
        assert np.array_equal(ha.offsets, hb.offsets) and np.array_equal(ha.keys, hb.keys)
        _download_matches(A, _expect(d, "pp1k", step)[0])


@pytest.mark.gpu
def test_device_apply_through_pool_growth_and_relayout(cuda, orc):
    """Rows that outgrow their slack move to the overflow pool; a batch larger
    than the pool forces a re-layout. Each step equals the oracle."""
    rng = np.random.default_rng(5)
    x = cuda.rmat(12, 8, seed=3)
    G = cuda.Graph(x)
    cur = x
    S = x.span
    for step in range(6):
        if step % 2 == 0:
            # concentrated: a few hubs gain many new neighbours (rows outgrow their room)
            hubs = rng.integers(1, S, 4).astype(np.uint32)
            n = 3000 * (step + 1)
            u = np.repeat(hubs, n // 4)
            v = rng.integers(1, S, len(u)).astype(np.uint32)
        else:
            # spread: many rows, most of the graph's size (outgrows the pool)
            n = cur.num_edges
            u = rng.integers(1, S, n).astype(np.uint32)
            v = rng.integers(1, S, n).astype(np.uint32)
        w = rng.integers(1, 4, len(u)).astype(np.float32)
        if step % 2 == 0:  # one direction: only the hub rows are touched
            ins = (u, v, w)
        else:
            ins = (np.concatenate([u, v]), np.concatenate([v, u]), np.concatenate([w, w]))
        deg = np.diff(cur.offsets).astype(np.int64)
        src = np.repeat(np.arange(S, dtype=np.uint32), deg)
        e = rng.choice(cur.num_edges, cur.num_edges // 20, replace=False)
        b = cuda.HostBatch(src[e], cur.keys[e], cur.weights[e], *ins)
        y, t = orc.apply_batch(cur, b)
        tb = G.apply_batch(b)
        _download_matches(G, y)
        assert _same(_tidy_tuple(tb), t)
        assert G.edge_weight() == orc.edge_weight(cuda.HostGraph(*y))
        cur = cuda.HostGraph(*y)


@pytest.mark.gpu
def test_methods_on_device_updated_graph_equal_fresh_upload(cuda):
    """Static and the three dynamic methods (deterministic mode) give the same
    result on a device-updated graph as on the same rows uploaded afresh."""
    x = cuda.planted_partition(4096, 128, 16, 0.8, 17)
    o = cuda.LouvainOptions(deterministic=True)
    G = cuda.Graph(x)
    r0 = cuda.louvain_static(G, o)
    b = cuda.random_batch(x, 2000, 0.8, seed=4)
    tb = G.apply_batch(b)
    F = cuda.Graph(G.download())
    for fn in (cuda.louvain_naive_dynamic, cuda.louvain_dynamic_delta_screening, cuda.louvain_dynamic_frontier):
        a = fn(G, tb, r0.membership, r0.vertexWeight, r0.communityWeight, o)
        c = fn(F, tb, r0.membership, r0.vertexWeight, r0.communityWeight, o)
        assert np.array_equal(a.membership, c.membership), fn.__name__
        assert (a.iterations, a.passes) == (c.iterations, c.passes)
    a, c = cuda.louvain_static(G, o), cuda.louvain_static(F, o)
    assert np.array_equal(a.membership, c.membership)


@pytest.mark.gpu
def test_apply_edge_cases(cuda):
    x = cuda.planted_partition(512, 32, 8, 0.8, 2)
    G = cuda.Graph(x)
    h0 = G.download()
    # empty batch: nothing changes
    t = G.apply_batch(cuda.HostBatch.empty())
    assert t.num_deletions == 0 and t.num_insertions == 0
    h1 = G.download()
    assert np.array_equal(h0.keys, h1.keys) and np.array_equal(h0.offsets, h1.offsets)
    # ids >= span are rejected before anything changes
    bad = cuda.HostBatch(np.zeros(0, np.uint32), np.zeros(0, np.uint32), np.zeros(0, np.float32),
                         np.array([1], np.uint32), np.array([x.span], np.uint32), np.ones(1, np.float32))
    with pytest.raises(cuda.LvgError) as e:
        G.apply_batch(bad)
    assert e.value.code == cuda.LVG_EINVAL
    assert np.array_equal(G.download().keys, h0.keys)
    # rows that were not uploaded sorted cannot take a batch
    off = np.array([0, 2, 3, 4], np.uint64)
    U = cuda.Graph(cuda.HostGraph(off, np.array([2, 1, 0, 0], np.uint32), np.ones(4, np.float32),
                                  np.ones(3, np.uint8)))
    with pytest.raises(cuda.LvgError) as e:
        U.apply_batch(cuda.HostBatch(np.zeros(0, np.uint32), np.zeros(0, np.uint32), np.zeros(0, np.float32),
                                     np.array([1], np.uint32), np.array([2], np.uint32), np.ones(1, np.float32)))
    assert e.value.code == cuda.LVG_EINVAL
