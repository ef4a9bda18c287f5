"""Graph unions: many graphs clustered by one static Louvain run
(lvg_graph_create_union + lvg_static_union), each graph with the reference's
pass driver for itself (inc/louvain.hxx:1180-1215).

The bar: every graph's result in the union equals lvg_static on that graph
alone — bit for bit in deterministic mode (membership, vertex and community
weights including the community array's tail from earlier levels,
iterations, passes, residual affected count), and at the same modularity in
asynchronous mode. The mix covers graphs that finish at different passes,
a graph without edges (never starts), absent vertices, isolated vertices
and hubs above degree 8192 (the chunked hub path).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _mix(lvg):
    gs = [
        lvg.planted_partition(3000, 64, 12, 0.85, seed=1),
        lvg.planted_partition(20000, 128, 16, 0.7, seed=2),
        lvg.rmat(12, 16, seed=3),
        lvg.planted_partition(700, 32, 8, 0.9, seed=4),
    ]
    # no edges at all: M = 0, the driver never starts
    gs.append(lvg.HostGraph(np.zeros(6, np.uint64), np.zeros(0, np.uint32), np.zeros(0, np.float32),
                            np.array([0, 1, 1, 1, 1], np.uint8)))
    # isolated vertices and a self-loop, vertex 0 absent
    src = np.array([1, 2, 2, 3, 5, 5, 6, 7], np.uint32)
    dst = np.array([2, 1, 3, 2, 6, 5, 5, 7], np.uint32)
    gs.append(lvg.csr_from_edges(9, src, dst))
    gs.append(lvg.rmat(10, 12, seed=5))
    return gs


def _alone(cuda, hg, o):
    G = cuda.Graph(hg)
    r = cuda.louvain_static(G, o)
    G.close()
    return r


def _same(a, b, i):
    assert np.array_equal(a.membership, b.membership), i
    assert np.array_equal(a.vertexWeight, b.vertexWeight), i
    assert np.array_equal(a.communityWeight, b.communityWeight), i
    assert (a.iterations, a.passes, a.affectedVertices) == (b.iterations, b.passes, b.affectedVertices), i


@pytest.mark.parametrize("opts", [dict(), dict(aggregationTolerance=0.8), dict(maxPasses=2, maxIterations=3),
                                  dict(colors=4, tolerance=1e-3)])
def test_deterministic_union_equals_each_graph_alone(cuda, opts):
    gs = _mix(cuda)
    o = cuda.LouvainOptions(deterministic=True, **opts)
    U = cuda.Graph.union([cuda.Graph(g) for g in gs])
    assert U.union_graphs == len(gs)
    rs = cuda.louvain_static_union(U, o)
    assert len(rs) == len(gs)
    for i, g in enumerate(gs):
        assert len(rs[i].membership) == g.span
        _same(rs[i], _alone(cuda, g, o), i)


def test_union_with_hubs(cuda, lvg):
    # R-MAT scale 16, edge factor 48: hubs above degree 8192 next to small graphs
    gs = [lvg.planted_partition(5000, 64, 10, 0.8, seed=11), lvg.rmat(16, 48, seed=77),
          lvg.planted_partition(9000, 100, 20, 0.75, seed=12)]
    o = cuda.LouvainOptions(deterministic=True)
    U = cuda.Graph.union([cuda.Graph(g) for g in gs])
    rs = cuda.louvain_static_union(U, o)
    for i, g in enumerate(gs):
        _same(rs[i], _alone(cuda, g, o), i)


def test_async_union_quality(cuda, orc):
    """Asynchronous mode: each graph's modularity in the union — the mean over
    3 union runs, as the reference's side is the mean over 5 of its racing
    runs — is within 0.005 of the mean of 5 runs of the oracle's OpenMP port
    on that graph alone (a 1K-vertex R-MAT graph's single runs spread by
    about that much)."""
    gs = _mix(cuda)[:4] + [_mix(cuda)[6]]
    U = cuda.Graph.union([cuda.Graph(g) for g in gs])
    runs = [cuda.louvain_static_union(U) for _ in range(3)]
    for i, g in enumerate(gs):
        q_union = float(np.mean([orc.modularity(g, rs[i].membership) for rs in runs]))
        ref = [orc.modularity(g, orc.louvain(g, 0, threads=8)[0]) for _ in range(5)]
        assert abs(q_union - np.mean(ref)) <= 0.005, (i, q_union, ref)


def test_union_is_static_only(cuda):
    gs = _mix(cuda)[:2]
    U = cuda.Graph.union([cuda.Graph(g) for g in gs])
    with pytest.raises(RuntimeError):
        cuda.louvain_static(U)
    b = cuda.HostBatch(np.zeros(0, np.uint32), np.zeros(0, np.uint32), np.zeros(0, np.float32),
                       np.array([1], np.uint32), np.array([2], np.uint32), np.ones(1, np.float32))
    with pytest.raises(RuntimeError):
        U.apply_batch(b)
    with pytest.raises(RuntimeError):
        cuda.Graph.union([U])


def test_deterministic_union_matches_cpu_replay(cuda, orc):
    """Each graph of a deterministic union against the oracle's CPU replay of
    the same rule on that graph alone, bit for bit."""
    gs = _mix(cuda)
    o = cuda.LouvainOptions(deterministic=True)
    U = cuda.Graph.union([cuda.Graph(g) for g in gs])
    rs = cuda.louvain_static_union(U, o)
    for i, g in enumerate(gs):
        m, vt, ct, info = orc.louvain(g, 0, threads=4, sync=True, colors=o.effective_colors())
        assert np.array_equal(rs[i].membership, m), i
        assert np.array_equal(rs[i].vertexWeight, vt), i
        assert np.array_equal(rs[i].communityWeight, ct), i
        assert (rs[i].iterations, rs[i].passes, rs[i].affectedVertices) == (
            info["iterations"], info["passes"], info["affectedVertices"]), i


def test_union_phase_replay(cuda):
    """The union's first local-moving phase is captured on the call that
    repeats the first one's configuration and replayed as one graph (a
    conditional while node over every graph's stop test) on later calls: the
    same results, fewer host synchronisations."""
    gs = _mix(cuda)
    o = cuda.LouvainOptions(deterministic=True)
    U = cuda.Graph.union([cuda.Graph(g) for g in gs])
    first = cuda.louvain_static_union(U, o)
    s0 = U.stats()["host_syncs"]
    for _ in range(2):
        again = cuda.louvain_static_union(U, o)
        for i in range(len(gs)):
            _same(again[i], first[i], i)
    assert U.stats()["host_syncs"] < s0
