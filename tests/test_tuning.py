"""Launch-shape tuning (lvg_tuning) and the autotuner (lvg_autotune).

The knobs other than frontier_colors change only how the local-moving work is
launched (hub chunk size, concurrent degree bins, fused small bins, blocks
per SM of the large-degree kernels, the degree bins' limits and so the tile
width and table capacity that serve each degree), so deterministic results
must not move when they change. The autotuner picks among them by time on the caller's
workload; its colour-class choice is guarded by modularity.
"""
import numpy as np
import pytest


def test_tuning_defaults(lvg):
    t = lvg.tuning_default()
    assert t == dict(frontier_colors=8, concurrent_bins=1, fused_small=0, hub_chunk=4096, big_blocks_per_sm=0,
                     frontier_max_fraction=1e-3, hub_tables=1, bin_max_degree=[0] * 12, level_graphs=1, small_regs=64)


@pytest.fixture(scope="module")
def hubcase(lvg):
    x = lvg.rmat(16, 48, seed=77)
    b = lvg.random_batch(x, 3000, 0.8, seed=78)
    return x, b, lvg.apply_batch(x, b)


@pytest.mark.gpu
def test_launch_knobs_keep_deterministic_results(cuda, hubcase):
    x, b, y = hubcase
    o = cuda.LouvainOptions(deterministic=True)
    r0 = cuda.louvain_static(cuda.Graph(x), o)
    Y = cuda.Graph(y)
    ref = cuda.louvain_dynamic_frontier(Y, b, r0.membership, r0.vertexWeight, r0.communityWeight, o)
    # degree-bin limits: every bin's degrees handed to the next bin; odd
    # limits; bin 9 emptied into bin 10 (with fused small bins as well)
    shifted = [0, 0, 4, 8, 16, 32, 64, 128, 256, 512, 0, 0]
    odd = [0, 2, 0, 12, 0, 40, 0, 200, 0, 1024, 0, 0]
    for knobs in [dict(hub_chunk=1024), dict(hub_chunk=16384, concurrent_bins=0), dict(fused_small=1),
                  dict(big_blocks_per_sm=1), dict(big_blocks_per_sm=3, hub_chunk=2048),
                  dict(bin_max_degree=shifted, fused_small=0, big_blocks_per_sm=0),
                  dict(bin_max_degree=shifted, fused_small=1), dict(bin_max_degree=odd, fused_small=0),
                  dict(bin_max_degree=[0] * 9 + [512], concurrent_bins=1), dict(level_graphs=0),
                  dict(level_graphs=1, bin_max_degree=[0] * 12), dict(fused_small=1, small_regs=64),
                  dict(fused_small=4, small_regs=32)]:
        cuda.set_tuning(Y, **knobs)
        r = cuda.louvain_dynamic_frontier(Y, b, r0.membership, r0.vertexWeight, r0.communityWeight, o)
        assert np.array_equal(r.membership, ref.membership), knobs
        assert np.array_equal(r.communityWeight, ref.communityWeight), knobs
        assert (r.iterations, r.passes, r.affectedVertices) == (ref.iterations, ref.passes, ref.affectedVertices)
        s = cuda.louvain_static(Y, o)
        assert np.array_equal(s.membership, cuda.louvain_static(cuda.Graph(y), o).membership), knobs


@pytest.mark.gpu
def test_invalid_tuning_is_rejected(cuda, hubcase):
    Y = cuda.Graph(hubcase[2])
    for bad in [dict(hub_chunk=100), dict(frontier_colors=0), dict(frontier_colors=65), dict(big_blocks_per_sm=-1),
                dict(frontier_max_fraction=2.0),
                dict(bin_max_degree=[0, 5]),             # beyond bin 1's reach (4)
                dict(bin_max_degree=[0, 0, 0, 3]),       # below bin 2's limit (8)
                dict(bin_max_degree=[0] * 10 + [100]),   # bin 10 ends at the hubs' threshold
                dict(bin_max_degree=[7]), dict(level_graphs=2), dict(small_regs=48)]:
        with pytest.raises(RuntimeError):
            cuda.set_tuning(Y, **bad)
    assert cuda.get_tuning(Y) == cuda.tuning_default()


@pytest.mark.gpu
def test_autotune_frontier(cuda, orc, hubcase):
    x, b, y = hubcase
    r0 = cuda.louvain_static(cuda.Graph(x))
    Y = cuda.Graph(y)
    prior = cuda.State(Y)
    prior.set(r0.membership, r0.vertexWeight, r0.communityWeight)
    out = cuda.State(Y)
    db = cuda.DeviceBatch(Y, b)
    q_default = orc.modularity(y, cuda.louvain_dynamic_frontier(Y, b, r0.membership, r0.vertexWeight,
                                                                 r0.communityWeight).membership)
    t, ms = cuda.autotune(Y, cuda.METHOD_FRONTIER, db, prior, repeats=2)
    assert ms > 0 and cuda.get_tuning(Y) == t
    assert t["hub_chunk"] in (2048, 4096, 8192, 16384) and t["frontier_colors"] in (8, 4, 2, 1)
    r = cuda.louvain_dynamic_frontier(Y, b, r0.membership, r0.vertexWeight, r0.communityWeight)
    assert orc.modularity(y, r.membership) >= q_default - 5e-3


@pytest.mark.gpu
def test_autotune_union_static(cuda, lvg):
    gs = [lvg.planted_partition(4000 + 1000 * i, 64, 12, 0.8, seed=30 + i) for i in range(6)]
    U = cuda.Graph.union([cuda.Graph(g) for g in gs])
    o = cuda.LouvainOptions(deterministic=True)
    ref = cuda.louvain_static_union(U, o)
    t, ms = cuda.autotune(U, cuda.METHOD_STATIC, o=o, repeats=1)
    assert ms > 0
    rs = cuda.louvain_static_union(U, o)
    for a, b in zip(rs, ref):
        assert np.array_equal(a.membership, b.membership)
