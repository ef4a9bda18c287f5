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


@pytest.mark.gpu
def test_server_coalescing_serves_the_union(cuda, orc):
    """With coalescing, queued requests of one graph run as one batch: every
    ticket completes, and the graph ends as after the batches one by one."""
    x = cuda.planted_partition(4000, 100, 12, 0.8, 9)
    seq = [cuda.reference_batch(x, 0, 300, seed=50 + k) for k in range(12)]  # insertion-only
    cur = x
    for b in seq:
        cur = cuda.HostGraph(*orc.apply_batch(cur, b)[0])
    G = cuda.Graph(x)
    sv = cuda.Server(workers=2, coalesce=1 << 20)
    gid = sv.add_graph(G)
    tickets = [sv.submit(gid, b) for b in seq]
    infos = [sv.wait(t) for t in tickets]
    assert all(i["status"] == 0 for i in infos)
    st = sv.stats()
    assert st["completed"] == len(seq)
    sv.drain()
    h = G.download()
    assert np.array_equal(h.offsets, cur.offsets) and np.array_equal(h.keys, cur.keys)
    sv.close()


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
