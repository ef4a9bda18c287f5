"""The serving loop (lvg_server): many graphs resident in HBM, batch-update
requests applied and answered concurrently.

A server runs, per request, what main.cxx:108-125 runs per batch — tidy and
apply the batch to the graph, then the dynamic method from the previous
result — so in deterministic mode a graph's final state must not depend on
what else the server was doing: the test interleaves requests for several
graphs through 4 workers and compares each graph's state, bit for bit, with
the same sequence run alone through lvg_graph_apply_device_batch +
lvg_run_resident. Admission control refuses a graph that would exceed the
HBM budget.
"""
import numpy as np
import pytest


def _graphs(lvg):
    return [lvg.planted_partition(3000, 100, 12, 0.8, 1), lvg.rmat(11, 8, seed=2), lvg.planted_partition(5000, 64, 8, 0.7, 3),
            lvg.rmat(12, 4, seed=4), lvg.planted_partition(1500, 150, 20, 0.9, 5)]


def _batches(lvg, orc, x, k, seed):
    """k untidy batches drawn one after another on the evolving graph."""
    out = []
    cur = x
    for j in range(k):
        b = lvg.reference_batch(cur, 40 + 10 * j, 200 + 50 * j, seed=seed * 100 + j)
        cur = lvg.HostGraph(*orc.apply_batch(cur, b)[0])
        out.append(b)
    return out


def test_footprint_grows_with_the_graph(lvg):
    lvg.load_library()
    assert lvg.graph_footprint(1000, 10_000) < lvg.graph_footprint(1000, 20_000) < lvg.graph_footprint(2000, 20_000)


@pytest.mark.gpu
def test_server_results_equal_sequential_runs(cuda, orc):
    o = cuda.LouvainOptions(deterministic=True)
    xs = _graphs(cuda)
    seqs = [_batches(cuda, orc, x, 4, i + 1) for i, x in enumerate(xs)]
    # alone
    alone = []
    for x, seq in zip(xs, seqs):
        G = cuda.Graph(x)
        st = cuda.State(G)
        cuda.run_resident(G, cuda.METHOD_STATIC, None, None, st, o)
        for b in seq:
            db = cuda.DeviceBatch(G, b)
            G.apply_batch(db)
            cuda.run_resident(G, cuda.METHOD_FRONTIER, db, st, st, o)
        alone.append(st.get())
    # served: requests interleaved across graphs
    sv = cuda.Server(workers=4, method=cuda.METHOD_FRONTIER, o=o)
    Gs = [cuda.Graph(x) for x in xs]
    ids = [sv.add_graph(G) for G in Gs]
    tickets = []
    for j in range(4):
        for gid, seq in zip(ids, seqs):
            tickets.append(sv.submit(gid, seq[j]))
    infos = [sv.wait(t) for t in tickets]
    assert all(i["status"] == 0 for i in infos)
    assert all(i["latency_ms"] >= i["run_ms"] for i in infos)
    for gid, ref in zip(ids, alone):
        m, vt, ct = sv.state(gid)
        assert np.array_equal(m, ref[0])
        assert np.array_equal(vt, ref[1]) and np.array_equal(ct, ref[2])
    st = sv.stats()
    assert st["completed"] == len(tickets) and st["failed"] == 0
    assert st["p99_ms"] >= st["p50_ms"] > 0
    sv.close()


@pytest.mark.gpu
def test_server_admission_control(cuda):
    """A graph is admitted on its measured device bytes; the next one that
    would pass the budget is refused with LVG_ENOMEM."""
    x = cuda.planted_partition(2000, 100, 10, 0.8, 1)
    G = cuda.Graph(x)
    probe = cuda.Server(workers=1)
    probe.add_graph(G)
    one = probe.stats()["hbm_reserved"]
    probe.close()
    assert one >= G.device_bytes() > 8 * x.num_edges
    H, K = cuda.Graph(x), cuda.Graph(x)
    sv = cuda.Server(workers=2, hbm_budget=one + one // 2)
    sv.add_graph(H)
    with pytest.raises(cuda.LvgError) as e:
        sv.add_graph(K)
    assert e.value.code == cuda.LVG_ENOMEM
    assert sv.stats()["graphs"] == 1
    sv.close()


def _edges(b):
    """Directed (src, dst) keys a batch deletes and inserts."""
    return (set(zip(b.del_src.tolist(), b.del_dst.tolist())), set(zip(b.ins_src.tolist(), b.ins_dst.tolist())))


def _conflict(earlier, b):
    """b touches an edge the earlier requests insert, or inserts one they delete."""
    dels, ins = set(), set()
    for e in earlier:
        d, i = _edges(e)
        dels |= d
        ins |= i
    d, i = _edges(b)
    return bool(d & ins) or bool(i & (ins | dels))


def _pair(lvg, u, v, w):
    return lvg.HostBatch(np.zeros(0, np.uint32), np.zeros(0, np.uint32), np.zeros(0, np.float32),
                         np.array([u, v], np.uint32), np.array([v, u], np.uint32), np.array([w, w], np.float32))


def _unpair(lvg, u, v, w):
    return lvg.HostBatch(np.array([u, v], np.uint32), np.array([v, u], np.uint32), np.array([w, w], np.float32),
                         np.zeros(0, np.uint32), np.zeros(0, np.uint32), np.zeros(0, np.float32))


def _union(lvg, bs):
    """The batch a coalesced group runs: deletions, then insertions, in arrival order."""
    cat = lambda f: np.concatenate([getattr(b, f) for b in bs])
    return lvg.HostBatch(cat("del_src"), cat("del_dst"), cat("del_w"), cat("ins_src"), cat("ins_dst"), cat("ins_w"))


@pytest.mark.gpu
def test_server_coalescing_serves_the_union(cuda, orc):
    """With coalescing, queued requests of one graph run as one batch, and a
    group ends before a request that conflicts with it: an edge inserted and
    then deleted, deleted and then inserted, or inserted twice with different
    weights. So the graph after all requests equals the graph after each
    request one by one (the reference's tidy + apply, weights included), and
    the memberships equal those of each group's union applied alone in the
    same order (deterministic mode, bit for bit)."""
    o = cuda.LouvainOptions(deterministic=True)
    x = cuda.planted_partition(6000, 100, 12, 0.8, 9)
    adj = [set(x.keys[x.offsets[u]:x.offsets[u + 1]].tolist()) for u in range(x.span)]
    rng = np.random.default_rng(3)
    free = []
    while len(free) < 2:
        u, v = (int(t) for t in rng.integers(1, x.span, 2))
        if u != v and v not in adj[u] and (u, v) not in free:
            free.append((u, v))
    (a, b), (c, d) = free
    # a long first request, so the rest queue up behind it and coalesce
    seq = [cuda.reference_batch(x, 2000, 8000, seed=40)]
    seq += [_pair(cuda, a, b, 1.0), _unpair(cuda, a, b, 1.0),   # insert, then delete
            _pair(cuda, c, d, 1.0), _pair(cuda, c, d, 2.0),     # insert twice, different weights
            _unpair(cuda, c, d, 1.0), _pair(cuda, c, d, 3.0)]   # delete, then insert again
    cur = x
    for b_ in seq:
        cur = cuda.HostGraph(*orc.apply_batch(cur, b_)[0])
    for k in range(6):
        nb = cuda.reference_batch(cur, 30, 120, seed=60 + k)
        seq.append(nb)
        cur = cuda.HostGraph(*orc.apply_batch(cur, nb)[0])
    G = cuda.Graph(x)
    sv = cuda.Server(workers=1, coalesce=1 << 20, o=o)
    gid = sv.add_graph(G)
    tickets = [sv.submit(gid, b_) for b_ in seq]
    infos = [sv.wait(t) for t in tickets]
    assert all(i["status"] == 0 for i in infos)
    assert sv.stats()["completed"] == len(seq)
    groups = {}
    for k, i in enumerate(infos):
        groups.setdefault(i["group"], []).append(k)
    order = sorted(groups)
    assert any(len(groups[g]) > 1 for g in order), "no request was coalesced"
    for g in order:
        ks = groups[g]
        assert ks == list(range(ks[0], ks[0] + len(ks)))          # consecutive requests
        assert all(infos[k]["coalesced"] == len(ks) for k in ks)
        for j in range(1, len(ks)):
            assert not _conflict([seq[k] for k in ks[:j]], seq[ks[j]])
    m, vt, ct = sv.state(gid)
    h = G.download()
    assert np.array_equal(h.offsets, cur.offsets) and np.array_equal(h.keys, cur.keys)
    assert np.array_equal(h.weights, cur.weights)
    sv.close()
    # each group's union, alone and in order, from the same static start
    R = cuda.Graph(x)
    st = cuda.State(R)
    cuda.run_resident(R, cuda.METHOD_STATIC, None, None, st, o)
    for g in order:
        db = cuda.DeviceBatch(R, _union(cuda, [seq[k] for k in groups[g]]))
        R.apply_batch(db)
        cuda.run_resident(R, cuda.METHOD_FRONTIER, db, st, st, o)
    rm, rvt, rct = st.get()
    assert np.array_equal(m, rm) and np.array_equal(vt, rvt) and np.array_equal(ct, rct)


@pytest.mark.gpu
def test_static_many_equals_one_by_one(cuda):
    o = cuda.LouvainOptions(deterministic=True)
    xs = _graphs(cuda)
    Gs = [cuda.Graph(x) for x in xs]
    many = cuda.louvain_static_many(Gs, o, workers=3, trim=2)
    for G, r in zip(Gs, many):
        one = cuda.louvain_static(G, o)
        assert np.array_equal(r["membership"], one.membership)
        assert (r["iterations"], r["passes"]) == (one.iterations, one.passes)
