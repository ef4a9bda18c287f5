"""The local-moving phase of the uploaded level replayed as one CUDA graph.

A handle's first call of a method runs the phase's first iteration on its own
(one synchronisation, for the reference's stop test el <= E,
inc/louvain.hxx:588-609) and the rest as a graph built for the call; a call
that repeats the previous call's configuration captures the whole phase as a
graph whose conditional while node evaluates that test on the device. Later calls with the
same level and options replay it: one launch and one synchronisation per
phase. The replay must give the per-iteration path's results: bit-exact with
the oracle's CPU replay in deterministic mode, on every call. A frontier call
that ends after its first pass waits for the GPU once.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FN = {1: "louvain_naive_dynamic", 2: "louvain_dynamic_delta_screening", 3: "louvain_dynamic_frontier"}


def prior(golden):
    return golden["static_m"], golden["static_vt"], golden["static_ct"]


@pytest.mark.parametrize("method", [0, 1, 2, 3])
def test_replayed_phase_matches_cpu_replay(cuda, orc, golden, method):
    o = cuda.LouvainOptions(deterministic=True)
    if method == 0:
        G = cuda.Graph(golden.x)
        m, vt, ct, info = orc.louvain(golden.x, 0, threads=4, sync=True, colors=o.effective_colors())
        call = lambda: cuda.louvain_static(G, o)  # noqa: E731
    else:
        G = cuda.Graph(golden.y)
        m, vt, ct, info = orc.louvain(golden.y, method, golden.b, *prior(golden), threads=4, sync=True,
                                      colors=o.effective_colors())
        call = lambda: getattr(cuda, FN[method])(G, golden.b, *prior(golden), o)  # noqa: E731
    syncs = []
    for _ in range(3):  # no capture, capture, replay
        r = call()
        syncs.append(G.stats()["host_syncs"])
        assert np.array_equal(r.membership, m)
        assert np.array_equal(r.vertexWeight, vt)
        assert np.array_equal(r.communityWeight, ct)
        assert (r.iterations, r.passes, r.affectedVertices) == (info["iterations"], info["passes"],
                                                                info["affectedVertices"])
    # a replayed first phase waits once however many iterations it ran
    assert syncs[2] <= syncs[0]


def test_replayed_async_phase_quality(cuda, orc, golden):
    """Asynchronous mode: every call, replayed or not, stays within 0.005 of
    the reference's mean modularity (the tolerance of the asynchronous parity
    tests)."""
    G = cuda.Graph(golden.y)
    for _ in range(3):
        r = cuda.louvain_dynamic_frontier(G, golden.b, *prior(golden))
        q = orc.modularity(golden.y, r.membership)
        assert abs(q - float(golden["df_q_mean8"])) <= 0.005, q
        ex = golden.y.exists.astype(bool)
        sums = np.zeros(golden.y.span)
        np.add.at(sums, r.membership[ex], r.vertexWeight[ex])
        live = np.unique(r.membership[ex])
        assert np.allclose(sums[live], r.communityWeight[live], rtol=0, atol=1e-9)


def test_resident_frontier_waits_once(cuda, golden):
    """A frontier run whose first pass ends the run (an empty batch: nothing
    to move) synchronises once when its phase is replayed: the residual
    affected count is read back by the same synchronisation."""
    Y = cuda.Graph(golden.y)
    st_prior, st_out = cuda.State(Y), cuda.State(Y)
    st_prior.set(*prior(golden))
    for batch in (cuda.HostBatch.empty(), golden.b):
        db = cuda.DeviceBatch(Y, batch)
        runs = [cuda.run_resident(Y, cuda.METHOD_FRONTIER, db, st_prior, st_out) for _ in range(3)]
        syncs = Y.stats()["host_syncs"]
        if runs[-1]["passes"] == 1:
            assert syncs == 1, (runs[-1], syncs)
        assert syncs >= 1
    m, vt, ct = st_out.get()
    ex = golden.y.exists.astype(bool)
    assert (m[ex] < golden.y.span).all()


@pytest.mark.parametrize("method", [0, 3])
def test_level_phase_graphs(cuda, orc, golden, method):
    """Aggregated levels: the iterations after a level's first run as one
    graph launch built for the level (lvg_tuning.level_graphs). Deterministic
    results equal the oracle's replay with the graphs on and off, and the
    graphs never add synchronisations."""
    o = cuda.LouvainOptions(deterministic=True)
    x = golden.x if method == 0 else golden.y
    if method == 0:
        m, vt, ct, info = orc.louvain(x, 0, threads=4, sync=True, colors=o.effective_colors())
    else:
        m, vt, ct, info = orc.louvain(x, method, golden.b, *prior(golden), threads=4, sync=True,
                                      colors=o.effective_colors())
    syncs, graphs = {}, {}
    for on in (1, 0, 1):
        G = cuda.Graph(x)
        cuda.set_tuning(G, level_graphs=on)
        r = cuda.louvain_static(G, o) if method == 0 else \
            cuda.louvain_dynamic_frontier(G, golden.b, *prior(golden), o)
        assert np.array_equal(r.membership, m), on
        assert np.array_equal(r.vertexWeight, vt), on
        assert np.array_equal(r.communityWeight, ct), on
        assert (r.iterations, r.passes, r.affectedVertices) == (info["iterations"], info["passes"],
                                                                info["affectedVertices"]), on
        st = G.stats()
        syncs[on], graphs[on] = st["host_syncs"], st["level_graphs"]
    assert graphs[0] == 0
    assert syncs[1] <= syncs[0], (syncs, graphs)


def test_level_phase_graphs_in_a_union(cuda, orc, lvg):
    """A graph union's aggregated levels run their later iterations as one
    graph too (the loop goes on while any graph still moves); each graph's
    deterministic result equals the oracle's replay of it alone."""
    gs = [lvg.planted_partition(3000 + 2000 * i, 48, 12, 0.75, seed=90 + i) for i in range(4)]
    o = cuda.LouvainOptions(deterministic=True)
    U = cuda.Graph.union([cuda.Graph(g) for g in gs])
    cuda.set_tuning(U, level_graphs=1)
    rs = cuda.louvain_static_union(U, o)
    assert U.stats()["level_graphs"] > 0
    for i, g in enumerate(gs):
        m, vt, ct, info = orc.louvain(g, 0, threads=4, sync=True, colors=o.effective_colors())
        assert np.array_equal(rs[i].membership, m), i
        assert np.array_equal(rs[i].communityWeight, ct), i
        assert (rs[i].iterations, rs[i].passes) == (info["iterations"], info["passes"]), i
