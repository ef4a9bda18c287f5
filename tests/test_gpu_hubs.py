"""The large-degree paths on the GPU: degree bins 9-10 (block per vertex,
shared tables with a global fallback) and bin 11 (hubs of degree > 8192:
chunked partial tables + merge), bit-exact against the CPU replay of the
deterministic rule.

The golden cases have no vertex above degree ~2000; an R-MAT graph of scale
16 with edge factor 48 (a = 0.57) has 17 hubs above degree 8192 (one above
16384, so several chunks) and ~120 vertices of degree 2049-8192, so every
local-moving path runs — including, in the first iteration of static
Louvain (every vertex its own community), chunks and vertices whose distinct
neighbour communities overflow the shared tables.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def hubgraph(lvg):
    x = lvg.rmat(16, 48, seed=77)
    deg = np.diff(x.offsets).astype(np.int64)
    assert (deg > 16384).sum() >= 1 and (deg > 8192).sum() >= 10 and ((deg > 2048) & (deg <= 8192)).sum() >= 50
    b = lvg.random_batch(x, 3000, 0.8, seed=78)
    y = lvg.apply_batch(x, b)
    return x, b, y


@pytest.mark.parametrize("colors", [4, 16])
def test_static_and_frontier_on_hubs_match_cpu_replay(cuda, orc, hubgraph, colors):
    x, b, y = hubgraph
    o = cuda.LouvainOptions(deterministic=True, colors=colors)
    X = cuda.Graph(x)
    r0 = cuda.louvain_static(X, o)
    m, vt, ct, info = orc.louvain(x, 0, threads=8, sync=True, colors=colors)
    assert np.array_equal(r0.membership, m)
    assert np.array_equal(r0.communityWeight, ct)
    assert (r0.iterations, r0.passes) == (info["iterations"], info["passes"])
    Y = cuda.Graph(y)
    r = cuda.louvain_dynamic_frontier(Y, b, r0.membership, r0.vertexWeight, r0.communityWeight, o)
    m, vt, ct, info = orc.louvain(y, 3, b, r0.membership, r0.vertexWeight, r0.communityWeight, threads=8, sync=True,
                                  colors=colors)
    assert np.array_equal(r.membership, m)
    assert np.array_equal(r.communityWeight, ct)
    assert (r.iterations, r.passes, r.affectedVertices) == (info["iterations"], info["passes"],
                                                            info["affectedVertices"])


TOL = 0.005  # |dQ| against the mean of 5 runs of the oracle's OpenMP port


def test_async_on_hubs_quality_and_totals(cuda, orc, hubgraph):
    x, b, y = hubgraph
    X = cuda.Graph(x)
    r0 = cuda.louvain_static(X)
    q_gpu = orc.modularity(x, r0.membership)
    qs = [orc.modularity(x, orc.louvain(x, 0, threads=8)[0]) for _ in range(5)]
    assert abs(q_gpu - np.mean(qs)) <= TOL, (q_gpu, qs)
    # the dynamic methods from the same (GPU) prior on the updated graph
    prior = (r0.membership, r0.vertexWeight, r0.communityWeight)
    Y = cuda.Graph(y)
    for method, fn in ((1, cuda.louvain_naive_dynamic), (2, cuda.louvain_dynamic_delta_screening),
                       (3, cuda.louvain_dynamic_frontier)):
        ref = [orc.modularity(y, orc.louvain(y, method, b, *prior, threads=8)[0]) for _ in range(5)]
        q = orc.modularity(y, fn(Y, b, *prior).membership)
        assert abs(q - np.mean(ref)) <= TOL, (method, q, ref)
    # the vertex weights are the weighted degrees (louvainVertexWeightsOmpW)
    deg_w = np.add.reduceat(x.weights.astype(np.float64), x.offsets[:-1].astype(np.int64)) * (np.diff(x.offsets) > 0)
    assert np.array_equal(r0.vertexWeight, deg_w)


def test_half_integer_weights_match_cpu_replay(cuda, orc, hubgraph):
    # Non-integer weights whose FP32 sums stay exact (multiples of 1/2 below
    # 2^23): the deterministic replay still matches bit for bit, hubs included.
    x, _, _ = hubgraph
    xh = type(x)(x.offsets, x.keys, (x.weights * 0.5).astype(np.float32), x.exists)
    o = cuda.LouvainOptions(deterministic=True, colors=16)
    r = cuda.louvain_static(cuda.Graph(xh), o)
    m, vt, ct, info = orc.louvain(xh, 0, threads=8, sync=True, colors=16)
    assert np.array_equal(r.membership, m)
    assert np.array_equal(r.communityWeight, ct)
    assert (r.iterations, r.passes) == (info["iterations"], info["passes"])


def test_delta_screening_on_hubs_matches_cpu_replay(cuda, orc, hubgraph):
    # The eight largest hubs each gain 20 edges, so the neighbour screening
    # runs over hub adjacencies (chunked over many blocks); flags and the
    # whole deterministic run equal the reference's.
    x, b, _ = hubgraph
    hubs = np.argsort(np.diff(x.offsets).astype(np.int64))[-8:]
    rng = np.random.default_rng(79)
    s, d = [], []
    for h in hubs:
        for v in rng.choice(np.arange(1, x.span), 20, replace=False):
            if v != h:
                s += [h, v]
                d += [v, h]
    ins_s = np.concatenate([b.ins_src, np.array(s, np.uint32)])
    ins_d = np.concatenate([b.ins_dst, np.array(d, np.uint32)])
    raw = cuda.HostBatch(b.del_src, b.del_dst, b.del_w, ins_s, ins_d, np.ones(len(ins_s), np.float32))
    o = cuda.LouvainOptions(deterministic=True)
    X = cuda.Graph(x)
    r0 = cuda.louvain_static(X, o)
    q = (r0.membership, r0.vertexWeight, r0.communityWeight)
    Y = X.clone()
    tb = Y.apply_batch(raw)
    y = Y.download()
    upd = cuda.louvain_dynamic_frontier(Y, tb, *q, cuda.LouvainOptions(maxPasses=0))
    v, n, c = cuda.affected_vertices(Y, cuda.METHOD_DELTA, tb, *q)
    rv, rn, rc = orc.ds_mark(y, tb, r0.membership, upd.vertexWeight, upd.communityWeight, Y.edge_weight() / 2)
    assert np.array_equal(v, rv) and np.array_equal(n, rn) and np.array_equal(c, rc)
    assert n[hubs].any()
    r = cuda.louvain_dynamic_delta_screening(Y, tb, *q, o)
    m, vt, ct, info = orc.louvain(y, 2, tb, *q, threads=8, sync=True)
    assert np.array_equal(r.membership, m)
    assert np.array_equal(r.communityWeight, ct)
    assert (r.iterations, r.passes, r.affectedVertices) == (info["iterations"], info["passes"],
                                                            info["affectedVertices"])
