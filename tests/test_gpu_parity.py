"""CUDA path (liblouvain_gb300.so, through the C-ABI) against the reference's
golden outputs and the oracle.

Bit-exact: weighted degrees, the batch weight update, DF/DS affected sets, the
aggregated graph for a given membership (row-sorted), and the deterministic
mode against the oracle's CPU replay of the same rule. Tolerance: modularity
of the asynchronous mode within 0.005 (absolute) of the reference's mean over
5 multi-threaded runs.
"""
import numpy as np
import pytest

from conftest import rows_sorted

pytestmark = pytest.mark.gpu

QTOL = 0.005  # modularity tolerance against the reference's mean


@pytest.fixture(scope="module")
def dev(cuda, golden):
    return cuda.Graph(golden.x), cuda.Graph(golden.y)


def prior(golden):
    return golden["static_m"], golden["static_vt"], golden["static_ct"]


def test_graph_properties(cuda, golden, dev):
    X, Y = dev
    assert X.span == golden.x.span and X.order == golden.x.order and X.size == golden.x.num_edges
    assert X.edge_weight() / 2 == golden["x_M"]
    assert Y.edge_weight() / 2 == golden["y_M"]


def test_vertex_weights_bit_exact(cuda, golden, dev):
    X, _ = dev
    r = cuda.louvain_static(X, cuda.LouvainOptions(maxPasses=0))
    assert np.array_equal(r.vertexWeight, golden["x_vtot"])
    assert np.array_equal(r.communityWeight, golden["x_vtot"])
    ex = golden.x.exists.astype(bool)
    ids = np.arange(golden.x.span, dtype=np.uint32)
    assert np.array_equal(r.membership[ex], ids[ex]) and np.all(r.membership[~ex] == 0)
    assert r.passes == 0 and r.iterations == 0


def test_vertex_and_community_weight_utilities(cuda, golden, dev):
    # louvainVertexWeightsOmpW and louvainCommunityWeightsOmpW through the C-ABI utilities
    X, _ = dev
    vt = X.vertex_weights()
    assert np.array_equal(vt, golden["x_vtot"])
    m = golden["static_m"]
    expect = np.bincount(m, weights=golden["x_vtot"], minlength=golden.x.span)
    assert np.array_equal(X.community_weights(m), expect)
    assert np.array_equal(X.community_weights(m, 2 * vt), 2 * expect)


def test_batch_weight_update_bit_exact(cuda, golden, dev):
    _, Y = dev
    r = cuda.louvain_dynamic_frontier(Y, golden.b, *prior(golden), cuda.LouvainOptions(maxPasses=0))
    assert np.array_equal(r.vertexWeight, golden["upd_vt"])
    assert np.array_equal(r.communityWeight, golden["upd_ct"])
    assert np.array_equal(r.membership, golden["static_m"])


def test_frontier_flags_bit_exact(cuda, golden, dev):
    _, Y = dev
    f = cuda.affected_vertices(Y, cuda.METHOD_FRONTIER, golden.b, *prior(golden))
    assert np.array_equal(f, golden["df_flags"])


def test_delta_screening_flags_bit_exact(cuda, golden, dev):
    _, Y = dev
    v, n, c = cuda.affected_vertices(Y, cuda.METHOD_DELTA, golden.b, *prior(golden))
    assert np.array_equal(v, golden["ds_vertices"])
    assert np.array_equal(n, golden["ds_neighbors"])
    assert np.array_equal(c, golden["ds_communities"])


def test_aggregation_bit_exact(cuda, golden, dev):
    _, Y = dev
    ren, CN, off, keys, w = cuda.aggregate(Y, golden["static_m"])
    assert CN == golden["agg_cn"]
    assert np.array_equal(ren, golden["agg_ren"])
    r, k, x = rows_sorted(CN, off, keys, w)
    assert np.array_equal(r, golden["agg_row"])
    assert np.array_equal(k, golden["agg_key"])
    assert np.array_equal(x, golden["agg_w"])


def test_modularity_fp64(cuda, golden, dev, orc):
    X, _ = dev
    m = golden["static_m"]
    assert X.modularity(m) == pytest.approx(float(golden["static_q"]), abs=1e-12)
    assert X.modularity(m) == pytest.approx(orc.modularity(golden.x, m), abs=1e-12)


def _det(cuda, orc, golden, dev, method, colors):
    X, Y = dev
    o = cuda.LouvainOptions(deterministic=True, colors=colors)
    if method == 0:
        r = cuda.louvain_static(X, o)
        m, vt, ct, info = orc.louvain(golden.x, 0, threads=4, sync=True, colors=colors)
    else:
        fn = {1: cuda.louvain_naive_dynamic, 2: cuda.louvain_dynamic_delta_screening,
              3: cuda.louvain_dynamic_frontier}[method]
        r = fn(Y, golden.b, *prior(golden), o)
        m, vt, ct, info = orc.louvain(golden.y, method, golden.b, *prior(golden), threads=4, sync=True,
                                      colors=colors)
    return r, (m, vt, ct, info)


@pytest.mark.parametrize("method", [0, 1, 2, 3])
@pytest.mark.parametrize("colors", [1, 4, 16])
def test_deterministic_mode_matches_cpu_replay(cuda, orc, golden, dev, method, colors):
    r, (m, vt, ct, info) = _det(cuda, orc, golden, dev, method, colors)
    assert np.array_equal(r.membership, m)
    assert np.array_equal(r.vertexWeight, vt)
    assert np.array_equal(r.communityWeight, ct)
    assert (r.iterations, r.passes, r.affectedVertices) == (info["iterations"], info["passes"],
                                                            info["affectedVertices"])


def test_deterministic_mode_is_reproducible(cuda, golden, dev):
    X, _ = dev
    o = cuda.LouvainOptions(deterministic=True, repeat=3)
    a = cuda.louvain_static(X, o)
    b = cuda.louvain_static(X, cuda.LouvainOptions(deterministic=True))
    assert np.array_equal(a.membership, b.membership)


@pytest.mark.parametrize("method,tag", [(0, "static"), (1, "nd"), (2, "ds"), (3, "df")])
def test_async_quality_within_tolerance(cuda, golden, dev, orc, method, tag):
    X, Y = dev
    if method == 0:
        r = cuda.louvain_static(X)
        q = orc.modularity(golden.x, r.membership)
    else:
        fn = {1: cuda.louvain_naive_dynamic, 2: cuda.louvain_dynamic_delta_screening,
              3: cuda.louvain_dynamic_frontier}[method]
        r = fn(Y, golden.b, *prior(golden))
        q = orc.modularity(golden.y, r.membership)
    assert abs(q - float(golden[f"{tag}_q_mean8"])) <= QTOL, (q, float(golden[f"{tag}_q_mean8"]))
    assert r.passes >= 1 and r.iterations >= r.passes


def test_async_community_totals_consistent(cuda, golden, dev):
    """Σ vertex weights of each final community == its total (integer weights: exact)."""
    X, _ = dev
    r = cuda.louvain_static(X)
    ex = golden.x.exists.astype(bool)
    sums = np.zeros(golden.x.span)
    np.add.at(sums, r.membership[ex], r.vertexWeight[ex])
    live = np.unique(r.membership[ex])
    assert np.array_equal(sums[live], r.communityWeight[live])


def test_resident_api_matches_host_api(cuda, golden, dev):
    _, Y = dev
    o = cuda.LouvainOptions(deterministic=True)
    ref = cuda.louvain_dynamic_frontier(Y, golden.b, *prior(golden), o)
    st_prior, st_out = cuda.State(Y), cuda.State(Y)
    st_prior.set(*prior(golden))
    db = cuda.DeviceBatch(Y, golden.b)
    info = cuda.run_resident(Y, cuda.METHOD_FRONTIER, db, st_prior, st_out, o)
    m, vt, ct = st_out.get()
    assert np.array_equal(m, ref.membership)
    assert np.array_equal(vt, ref.vertexWeight) and np.array_equal(ct, ref.communityWeight)
    assert info["iterations"] == ref.iterations and info["passes"] == ref.passes
    # in place: prior == out
    st_prior.set(*prior(golden))
    cuda.run_resident(Y, cuda.METHOD_FRONTIER, db, st_prior, st_prior, o)
    assert np.array_equal(st_prior.get()[0], ref.membership)


def test_result_into_caller_buffers(cuda, golden, dev):
    X, _ = dev
    S = golden.x.span
    bufs = (cuda.PinnedArray(S, np.uint32), cuda.PinnedArray(S, np.float64), cuda.PinnedArray(S, np.float64))
    o = cuda.LouvainOptions(deterministic=True)
    r = cuda.louvain_static(X, o, out_buffers=tuple(b.array for b in bufs))
    r2 = cuda.louvain_static(X, o)
    assert np.array_equal(bufs[0].array, r2.membership) and np.array_equal(bufs[2].array, r2.communityWeight)
    assert r.passes == r2.passes


def test_invalid_inputs_rejected(cuda, golden, dev):
    _, Y = dev
    S = golden.y.span
    q, vt, ct = prior(golden)
    bad = cuda.HostBatch(np.array([S], np.uint32), np.array([1], np.uint32), np.ones(1, np.float32),
                         *[a.copy() for a in (golden.b.ins_src, golden.b.ins_dst, golden.b.ins_w)])
    with pytest.raises(cuda.LvgError) as e:
        cuda.louvain_dynamic_frontier(Y, bad, q, vt, ct)
    assert e.value.code == cuda.LVG_EINVAL
    badq = q.copy()
    badq[1] = S
    with pytest.raises(cuda.LvgError) as e:
        cuda.louvain_naive_dynamic(Y, golden.b, badq, vt, ct)
    assert e.value.code == cuda.LVG_EINVAL
    if golden.b.num_insertions > 1:
        rev = cuda.HostBatch(golden.b.del_src, golden.b.del_dst, golden.b.del_w, golden.b.ins_src[::-1].copy(),
                             golden.b.ins_dst[::-1].copy(), golden.b.ins_w[::-1].copy())
        with pytest.raises(cuda.LvgError) as e:
            cuda.louvain_dynamic_delta_screening(Y, rev, q, vt, ct)
        assert e.value.code == cuda.LVG_EINVAL


def test_empty_batch_and_empty_graph(cuda, golden, dev):
    _, Y = dev
    r = cuda.louvain_dynamic_frontier(Y, cuda.HostBatch.empty(), *prior(golden))
    assert r.passes >= 1
    S = 10
    e = cuda.HostGraph(np.zeros(S + 1, np.uint64), np.zeros(0, np.uint32), np.zeros(0, np.float32),
                       np.r_[0, np.ones(S - 1)].astype(np.uint8))
    G = cuda.Graph(e)
    r = cuda.louvain_static(G)
    assert r.passes == 0 and r.iterations == 0
    assert r.membership.tolist() == [0] + list(range(1, S))


def test_pinned_result_buffers_match(cuda, golden, dev):
    # Into pinned result arrays the vertex weights are copied out on a side
    # stream during the run; the results must equal those into pageable arrays.
    _, Y = dev
    S = golden.y.span
    o = cuda.LouvainOptions(deterministic=True)
    ref = cuda.louvain_dynamic_frontier(Y, golden.b, *prior(golden), o)
    bufs = [cuda.PinnedArray(S, np.uint32), cuda.PinnedArray(S, np.float64), cuda.PinnedArray(S, np.float64)]
    for _ in range(2):
        r = cuda.louvain_dynamic_frontier(Y, golden.b, *prior(golden), o, out_buffers=[b.array for b in bufs])
        assert np.array_equal(r.membership, ref.membership)
        assert np.array_equal(r.vertexWeight, ref.vertexWeight)
        assert np.array_equal(r.communityWeight, ref.communityWeight)


def test_delta_screening_flags_with_large_source_groups(cuda, orc):
    # Sources with more than 32 inserted edges take the block path of the
    # insertion screening, the others the warp path; both equal the reference.
    x = cuda.planted_partition(3000, 64, 10, 0.8, seed=21)
    rb = cuda.random_batch(x, 400, 0.8, seed=22)
    rng = np.random.default_rng(23)
    extra_s, extra_d = [], []
    # 1500 insertions: the per-block HBM table; 120, 40, 33: the shared one; 32: a warp
    for src, k in ((1, 120), (2, 40), (3, 33), (4, 32), (5, 1500)):
        for v in rng.choice(np.arange(6, 3001), k, replace=False):
            extra_s += [src, v]
            extra_d += [v, src]
    raw = cuda.HostBatch(rb.del_src, rb.del_dst, rb.del_w,
                         np.concatenate([rb.ins_src, np.array(extra_s, np.uint32)]),
                         np.concatenate([rb.ins_dst, np.array(extra_d, np.uint32)]),
                         np.ones(len(rb.ins_src) + len(extra_s), np.float32))
    X = cuda.Graph(x)
    p = cuda.louvain_static(X, cuda.LouvainOptions(deterministic=True))
    Y = X.clone()
    tb = Y.apply_batch(raw)
    q = (p.membership, p.vertexWeight, p.communityWeight)
    upd = cuda.louvain_dynamic_frontier(Y, tb, *q, cuda.LouvainOptions(maxPasses=0))
    v, n, c = cuda.affected_vertices(Y, cuda.METHOD_DELTA, tb, *q)
    rv, rn, rc = orc.ds_mark(Y.download(), tb, p.membership, upd.vertexWeight, upd.communityWeight,
                             Y.edge_weight() / 2)
    assert np.array_equal(v, rv) and np.array_equal(n, rn) and np.array_equal(c, rc)
    assert n[1] or n[2] or n[3] or n[5] or c.any()  # the large groups were screened


@pytest.mark.parametrize("scale", [1.0, 2.0 ** -10, 1e-20, 1e20])
@pytest.mark.parametrize("swap", [False, True])
def test_delta_screening_exact_tie_takes_first_community(cuda, orc, swap, scale):
    # Three 5-cliques (vertices 1-5, 6-10, 11-15); vertex 11 gains one edge
    # into each of the other two, whose totals are equal: the gains tie
    # exactly, the FP32 screen cannot separate them, and the reference's FP64
    # rule gives the community of the first insertion in batch order (to
    # vertex 3), whichever of the two community ids is smaller. Every weight
    # is `scale`: at 1e-20 and 1e20 the total weight is outside the FP32
    # screen's range and every source takes the FP64 rule.
    src, dst = [], []
    for base in (1, 6, 11):
        for a in range(base, base + 5):
            for b in range(base, base + 5):
                if a != b:
                    src.append(a)
                    dst.append(b)
    # span 17: the edge-list reader makes vertices 0..16 (16 isolated)
    x = cuda.csr_from_edges(16, np.array(src, np.uint32), np.array(dst, np.uint32),
                            np.full(len(src), scale, np.float32))
    la, lb = (6, 1) if swap else (1, 6)
    q = np.array([0] + [la] * 5 + [lb] * 5 + [11] * 5 + [16], np.uint32)
    sw = float(np.float32(scale))
    vt = np.array([0] + [4.0 * sw] * 15 + [0])
    ct = np.zeros(17)
    ct[[1, 6, 11]] = 20.0 * sw
    ins = [(3, 11), (8, 11), (11, 3), (11, 8)]
    e = np.zeros(0, np.uint32)
    raw = cuda.HostBatch(e, e, np.zeros(0, np.float32), np.array([a for a, _ in ins], np.uint32),
                         np.array([b for _, b in ins], np.uint32), np.full(4, scale, np.float32))
    Y = cuda.Graph(x)
    tb = Y.apply_batch(raw)
    upd = cuda.louvain_dynamic_frontier(Y, tb, q, vt, ct, cuda.LouvainOptions(maxPasses=0))
    v, n, c = cuda.affected_vertices(Y, cuda.METHOD_DELTA, tb, q, upd.vertexWeight, upd.communityWeight)
    rv, rn, rc = orc.ds_mark(Y.download(), tb, q, upd.vertexWeight, upd.communityWeight, Y.edge_weight() / 2)
    assert np.array_equal(v, rv) and np.array_equal(n, rn) and np.array_equal(c, rc)
    assert n[11] and c[la] and not c[lb]


def test_delta_screening_flags_with_fractional_weights(cuda, orc):
    # Weights in (0, 1] from a hash of each unordered pair, on the graph and
    # the batch: the FP32 screen of the insertion gains meets close
    # candidates and near-zero gains at varied magnitudes; its flags must
    # still equal the reference's FP64 rule.
    x = cuda.planted_partition(20000, 100, 12, 0.7, seed=31)
    # symmetric weights: a hash of the unordered pair
    src = np.repeat(np.arange(x.span, dtype=np.uint64), np.diff(x.offsets).astype(np.int64))
    lo = np.minimum(src, x.keys.astype(np.uint64))
    hi = np.maximum(src, x.keys.astype(np.uint64))
    h = (lo * np.uint64(2654435761) + hi * np.uint64(40503)) % np.uint64(1000003)
    x = cuda.HostGraph(x.offsets, x.keys, (0.05 + 0.95 * h / 1000003.0).astype(np.float32), x.exists)
    rb = cuda.random_batch(x, 6000, 0.8, seed=33)
    a, b = rb.ins_src.astype(np.uint64), rb.ins_dst.astype(np.uint64)
    hb = (np.minimum(a, b) * np.uint64(40503) + np.maximum(a, b) * np.uint64(2654435761)) % np.uint64(999983)
    raw = cuda.HostBatch(rb.del_src, rb.del_dst, rb.del_w, rb.ins_src, rb.ins_dst,
                         (0.01 + 0.99 * hb / 999983.0).astype(np.float32))
    X = cuda.Graph(x)
    p = cuda.louvain_static(X)
    Y = X.clone()
    tb = Y.apply_batch(raw)
    q = (p.membership, p.vertexWeight, p.communityWeight)
    upd = cuda.louvain_dynamic_frontier(Y, tb, *q, cuda.LouvainOptions(maxPasses=0))
    v, n, c = cuda.affected_vertices(Y, cuda.METHOD_DELTA, tb, *q)
    rv, rn, rc = orc.ds_mark(Y.download(), tb, p.membership, upd.vertexWeight, upd.communityWeight,
                             Y.edge_weight() / 2)
    assert np.array_equal(v, rv) and np.array_equal(n, rn) and np.array_equal(c, rc)
    assert n.sum() > 100
