"""The oracle against the reference's own code on fresh inputs, where the
harness over the reference's headers is built (oracle/_ref/, from the
checkout or from the headers staged beside the tree; skipped elsewhere).

The golden fixtures pin the oracle on three graphs. Here the same 1-thread
comparison — bit for bit: membership, vertex and community weights,
iterations, passes, residual affected count — runs on a sweep of seeded
graphs the fixtures do not hold: planted partitions and R-MAT graphs of
several sizes, with unit, dyadic and arbitrary FP32 edge weights, for the
four entry points from the reference's own static result, plus the batch
weight update, the DF and DS affected sets and one aggregation step; untidy
batches tidied and applied three in a row; and the base graph of a temporal
stream (the reader and CSR build of the package's
host library against readTemporalOmpW + symmetrizeOmp).
"""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def ref(lvg):
    from oracle import oracle as O

    O.build(ref=None)
    if not O.reference_available():
        pytest.skip("the harness over the reference's headers is not built here")
    r = O.Reference()
    r.threads(1)
    return r


def _weighted(lvg, g, kind, seed):
    """g with symmetric edge weights: unit, dyadic (0.5 steps) or arbitrary FP32."""
    if kind == "unit":
        return g
    S = g.span
    src = np.repeat(np.arange(S, dtype=np.uint64), np.diff(g.offsets).astype(np.int64))
    a, b = np.minimum(src, g.keys), np.maximum(src, g.keys)
    h = (a * 2654435761 + b * 40503 + seed) % 1000003  # the same for (u, v) and (v, u)
    w = (1 + (h % 6) * 0.5) if kind == "dyadic" else (0.05 + (h % 99991) / 99991.0 * 3.0)
    return lvg.HostGraph(g.offsets, g.keys, w.astype(np.float32), g.exists)


def _batch_weights(lvg, b, kind, seed):
    if kind == "unit":
        return b

    def w(s, d):
        a, c = np.minimum(s, d).astype(np.uint64), np.maximum(s, d).astype(np.uint64)
        h = (a * 2654435761 + c * 40503 + seed) % 1000003
        return ((1 + (h % 6) * 0.5) if kind == "dyadic" else (0.05 + (h % 99991) / 99991.0 * 3.0)).astype(np.float32)

    return lvg.HostBatch(b.del_src, b.del_dst, w(b.del_src, b.del_dst), b.ins_src, b.ins_dst,
                         w(b.ins_src, b.ins_dst))


CASES = [("pp", 1500, 7, "unit"), ("pp", 4000, 8, "dyadic"), ("pp", 2500, 9, "float"),
         ("rmat", 10, 10, "unit"), ("rmat", 11, 11, "dyadic"), ("rmat", 12, 12, "float")]


def _case(lvg, kind, size, seed, wkind):
    x = (lvg.planted_partition(size, 64, 12, 0.8, seed) if kind == "pp" else lvg.rmat(size, 12, seed=seed))
    x = _weighted(lvg, x, wkind, seed)
    b = lvg.random_batch(x, max(4, x.num_edges // 2 // 200), 0.8, seed=seed + 1)
    if b.num_deletions:  # deletions carry the graph's own weights
        S = x.span
        lookup = {}
        src = np.repeat(np.arange(S, dtype=np.uint32), np.diff(x.offsets).astype(np.int64))
        for u, v, w in zip(src, x.keys, x.weights):
            lookup[(int(u), int(v))] = w
        dw = np.array([lookup[(int(u), int(v))] for u, v in zip(b.del_src, b.del_dst)], np.float32)
        ins = _batch_weights(lvg, b, wkind, seed)
        b = lvg.HostBatch(b.del_src, b.del_dst, dw, ins.ins_src, ins.ins_dst, ins.ins_w)
    y = lvg.apply_batch(x, b)
    return x, b, y


def _same_run(a, b, what):
    assert np.array_equal(a[0], b[0]), what
    assert np.array_equal(a[1], b[1]), what
    assert np.array_equal(a[2], b[2]), what
    for k in ("iterations", "passes", "affectedVertices"):
        assert a[3][k] == b[3][k], (what, k, a[3][k], b[3][k])


@pytest.mark.parametrize("kind,size,seed,wkind", CASES)
def test_oracle_equals_reference_one_thread(lvg, orc, ref, kind, size, seed, wkind):
    x, b, y = _case(lvg, kind, size, seed, wkind)
    rx, ry = ref.graph(x), ref.graph(y)
    assert orc.edge_weight(x) == rx.edge_weight()
    assert np.array_equal(orc.vertex_weights(x), rx.vertex_weights())
    s_ref = rx.louvain(0)
    _same_run(orc.louvain(x, 0, threads=1), s_ref, (kind, size, "static"))
    q, vt, ct = s_ref[0], s_ref[1], s_ref[2]
    # the pieces the dynamic methods start from
    o_w, r_w = orc.update_weights(b, q, vt, ct), ry.update_weights(b, q, vt, ct)
    assert np.array_equal(o_w[0], r_w[0]) and np.array_equal(o_w[1], r_w[1])
    f = orc.df_mark(y.span, b, q)
    assert f.any() and np.array_equal(f, ry.df_mark(b, q))
    M = ry.edge_weight() / 2  # the updated graph's, as louvainDynamicDeltaScreeningOmp passes it
    for a, c in zip(orc.ds_mark(y, b, q, r_w[0], r_w[1], M), ry.ds_mark(b, q, r_w[0], r_w[1], M)):
        assert np.array_equal(a, c)
    for meth, name in ((1, "nd"), (2, "ds"), (3, "df")):
        _same_run(orc.louvain(y, meth, b, q, vt, ct, threads=1), ry.louvain(meth, b, q, vt, ct),
                  (kind, size, name))


@pytest.mark.parametrize("kind,size,seed,wkind", CASES[::2])
def test_oracle_aggregation_equals_reference(lvg, orc, ref, kind, size, seed, wkind):
    x, _, _ = _case(lvg, kind, size, seed, wkind)
    q = ref.graph(x).louvain(0)[0]
    ren_o, cn_o, rows_o = orc.aggregate(x, q)
    ren_r, cn_r, rows_r = ref.graph(x).aggregate(q)
    assert cn_o == cn_r and np.array_equal(ren_o, ren_r)
    assert rows_o == rows_r  # each super-vertex's row: neighbour community -> weight


@pytest.mark.parametrize("rows,lines,communities,seed", [(500, 4000, 10, 3), (2000, 9000, 40, 4)])
def test_temporal_base_graph_equals_reference(lvg, ref, tmp_path, rows, lines, communities, seed):
    """The base graph main.cxx builds from the first 90 % of a temporal
    stream (readTemporalOmpW + symmetrizeOmp), from the reference and from
    the host reader + CSR build, on streams with repeated lines, self-loops
    and ids at the row limit."""
    src, dst, _ = lvg.temporal_drift(rows, communities, lines, seed=seed)
    rng = np.random.default_rng(seed)
    k = rng.choice(lines, lines // 20, replace=False)
    src[k[: len(k) // 2]] = dst[k[: len(k) // 2]]              # self-loops
    src[k[len(k) // 2:]] = src[(k[len(k) // 2:] + 1) % lines]  # repeats of the next line's source
    dst[k[len(k) // 2:]] = dst[(k[len(k) // 2:] + 1) % lines]
    src[0], dst[0] = rows, 1                                   # the largest id
    path = str(tmp_path / "t.txt")
    lvg.write_temporal(path, src, dst)
    n = int(0.9 * lines)
    off, key, w, ex = ref.read_temporal(path, rows, n)
    r = lvg.TemporalReader(path)
    s, t, wt = r.read(n, symmetric=True)
    r.close()
    x = lvg.csr_from_edges(rows, s, t, wt)
    assert np.array_equal(x.offsets, off) and np.array_equal(x.keys, key)
    assert np.array_equal(x.weights, w) and np.array_equal(x.exists, ex)


def _untidy_batch(lvg, x, n, seed):
    """About 3n entries in random order: deletions of present and absent
    edges (some twice), insertions of new and present edges and of edges
    touching absent slots (some twice). A repeated entry repeats its weight,
    so the reference's unstable sort cannot make the result depend on which
    copy survives."""
    rng = np.random.default_rng(seed)
    S = x.span
    src = np.repeat(np.arange(S, dtype=np.uint32), np.diff(x.offsets).astype(np.int64))
    n = min(n, x.num_edges)
    e = rng.choice(x.num_edges, n, replace=False)
    a = rng.integers(0, S, (n // 3, 2)).astype(np.uint32)
    ds = np.concatenate([src[e], a[:, 0], src[e[: n // 6]]])
    dd = np.concatenate([x.keys[e], a[:, 1], x.keys[e[: n // 6]]])
    dw = np.concatenate([x.weights[e], np.ones(n // 3, np.float32), x.weights[e[: n // 6]]])
    r = rng.integers(0, S, (n, 2)).astype(np.uint32)
    rw = rng.integers(1, 6, n).astype(np.float32) * 0.75
    e2 = rng.choice(x.num_edges, max(n // 4, 1), replace=False)
    is_ = np.concatenate([r[:, 0], src[e2], r[: n // 5, 0]])
    id_ = np.concatenate([r[:, 1], x.keys[e2], r[: n // 5, 1]])
    iw = np.concatenate([rw, np.full(len(e2), 9.0, np.float32), rw[: n // 5]])
    p, q = rng.permutation(len(ds)), rng.permutation(len(is_))
    return lvg.HostBatch(ds[p].copy(), dd[p].copy(), dw[p].copy(), is_[q].copy(), id_[q].copy(), iw[q].copy())


@pytest.mark.parametrize("kind,size,seed", [("pp", 800, 31), ("rmat", 9, 32), ("pp", 3000, 33)])
def test_untidy_batch_apply_equals_reference(lvg, orc, ref, kind, size, seed):
    """tidyBatchUpdateU + applyBatchUpdateOmpU (the reference, in place on its
    DiGraph) against the oracle's restatement, three batches in a row: the
    graph after each and the tidied batch, bit for bit."""
    x = (lvg.planted_partition(size, 32, 8, 0.8, seed) if kind == "pp" else lvg.rmat(size, 8, seed=seed))
    rg = ref.graph(x)
    for step in range(3):
        b = _untidy_batch(lvg, x, max(8, x.num_edges // 40), seed * 10 + step)
        (yo, yk, yw, yex), t_ref = rg.apply_batch(b)
        (oo, ok, ow, oex), t_orc = orc.apply_batch(x, b)
        assert np.array_equal(yo, oo) and np.array_equal(yk, ok), (kind, step)
        assert np.array_equal(yw, ow) and np.array_equal(yex, oex), (kind, step)
        assert all(np.array_equal(a, c) for a, c in zip(t_ref, t_orc)), (kind, step)
        assert len(t_ref[0]) < b.num_deletions and len(t_ref[3]) < b.num_insertions  # tidying removed some
        x = lvg.HostGraph(oo, ok, ow, oex)
