"""Generate the golden fixtures of tests/golden/ from the reference's own code.

Run where the reference checkout is available (it compiles
oracle/ref_harness.cxx against the reference's unmodified headers):

    LVG_REFERENCE_DIR=<reference checkout> python tests/golden/make_golden.py

Every expected value below comes from a call into the reference harness
(oracle/_ref/libref_louvain.so): weighted degrees, the batch weight update,
the DF and DS affected sets, one aggregation step, the 1-thread runs of the
four entry points (deterministic: the reference's sweep is sequential with one
thread) and the mean modularity of 5 multi-threaded runs. The inputs are
seeded synthetic graphs from liblvg_graphgen.so plus one hand-made graph with
self-loops, absent vertices, isolated vertices and integer weights.

apply.npz holds the batch-update fixtures: untidy batches (unsorted, with
duplicates, deletions of absent edges, insertions of present edges and of
edges touching absent vertices) run through the reference's
tidyBatchUpdateU + applyBatchUpdateOmpU, twice in a row; the graphs after
each batch and the tidied batches. temporal.npz holds a temporal stream and the
base graph main.cxx builds from it. `--only apply` regenerates just these two.
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "louvain-communities-openmp-dynamic_gb300"))
sys.path.insert(0, ROOT)

import lvg  # noqa: E402
import lvg_build  # noqa: E402
from oracle import oracle as O  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def edge_case_graph() -> lvg.HostGraph:
    """60 slots; slots 0, 7 and 13 absent; 50..59 isolated; self-loops; weights 1..3."""
    S = 60
    rng = np.random.default_rng(1234)
    exists = np.ones(S, np.uint8)
    exists[[0, 7, 13]] = 0
    live = [u for u in range(1, 50) if exists[u]]
    und = {}
    # three dense groups plus sparse cross links
    groups = [live[:15], live[15:30], live[30:]]
    for g in groups:
        for i, u in enumerate(g):
            for v in g[i + 1:]:
                if rng.random() < 0.45:
                    und[(u, v)] = float(rng.integers(1, 4))
    for _ in range(25):
        u, v = rng.choice(live, 2, replace=False)
        und[(min(u, v), max(u, v))] = float(rng.integers(1, 4))
    for u in live[::6]:
        und[(u, u)] = 2.0  # self-loops
    rows = [dict() for _ in range(S)]
    for (u, v), w in und.items():
        rows[u][v] = w
        rows[v][u] = w
    off = np.zeros(S + 1, np.uint64)
    keys, ws = [], []
    for u in range(S):
        for v in sorted(rows[u]):
            keys.append(v)
            ws.append(rows[u][v])
        off[u + 1] = len(keys)
    return lvg.HostGraph(off, np.array(keys, np.uint32), np.array(ws, np.float32), exists)


def edge_case_batch(x: lvg.HostGraph) -> lvg.HostBatch:
    """Deletions of a few existing edges (incl. a self-loop), insertions touching isolated vertices."""
    dels, ins = [], []
    for u in (1, 16, 31):
        v = int(x.keys[x.offsets[u]])
        dels.append((u, v, float(x.weights[x.offsets[u]])))
    for (u, v, w) in [(2, 50, 1.0), (50, 51, 2.0), (3, 40, 3.0), (20, 45, 1.0), (52, 52, 1.0), (4, 33, 2.0)]:
        ins.append((u, v, w))

    def both(lst):
        out = set()
        for u, v, w in lst:
            out.add((u, v, w))
            out.add((v, u, w))
        return sorted(out)

    d, i = both(dels), both(ins)
    a = lambda lst, k, dt: np.array([t[k] for t in lst], dt)  # noqa: E731
    return lvg.HostBatch(a(d, 0, np.uint32), a(d, 1, np.uint32), a(d, 2, np.float32),
                         a(i, 0, np.uint32), a(i, 1, np.uint32), a(i, 2, np.float32))


def messy_batch(x: lvg.HostGraph, n: int, seed: int) -> lvg.HostBatch:
    """An untidy batch of about 3n entries. Duplicates repeat the weight of
    their first occurrence, so the reference's unstable sort cannot change
    the result."""
    rng = np.random.default_rng(seed)
    S = x.span
    src = np.repeat(np.arange(S, dtype=np.uint32), np.diff(x.offsets).astype(np.int64))
    n = min(n, x.num_edges)
    e = rng.choice(x.num_edges, n, replace=False)
    a = rng.integers(0, S, (n // 4, 2)).astype(np.uint32)               # mostly absent edges
    ds = np.concatenate([src[e], a[:, 0], src[e[: n // 8]]])
    dd = np.concatenate([x.keys[e], a[:, 1], x.keys[e[: n // 8]]])
    dw = np.concatenate([x.weights[e], np.ones(n // 4, np.float32), x.weights[e[: n // 8]]])
    r = rng.integers(0, S, (n, 2)).astype(np.uint32)                    # mostly new edges
    e2 = rng.choice(x.num_edges, max(n // 4, 1), replace=False)         # present edges
    rw = rng.integers(1, 5, n).astype(np.float32)
    is_ = np.concatenate([r[:, 0], src[e2], r[: n // 8, 0]])
    id_ = np.concatenate([r[:, 1], x.keys[e2], r[: n // 8, 1]])
    iw = np.concatenate([rw, rng.integers(5, 9, len(e2)).astype(np.float32), rw[: n // 8]])
    p, q = rng.permutation(len(ds)), rng.permutation(len(is_))
    return lvg.HostBatch(ds[p].copy(), dd[p].copy(), dw[p].copy(), is_[q].copy(), id_[q].copy(), iw[q].copy())


def apply_fixtures(ref) -> None:
    d = {}
    for name, x, n in (("pp1k", lvg.planted_partition(1024, 64, 12, 0.8, 21), 300),
                       ("edge", edge_case_graph(), 40)):
        rg = ref.graph(x)
        d.update({f"{name}_x_off": x.offsets, f"{name}_x_key": x.keys, f"{name}_x_w": x.weights,
                  f"{name}_x_ex": x.exists})
        for step in (1, 2):
            b = messy_batch(x, n, seed=100 * step + len(name))
            (yo, yk, yw, yex), tidy = rg.apply_batch(b)
            p = f"{name}_{step}_"
            d.update({p + "b_ds": b.del_src, p + "b_dd": b.del_dst, p + "b_dw": b.del_w,
                      p + "b_is": b.ins_src, p + "b_id": b.ins_dst, p + "b_iw": b.ins_w,
                      p + "y_off": yo, p + "y_key": yk, p + "y_w": yw, p + "y_ex": yex})
            d.update({p + "t_" + k: v for k, v in zip(("ds", "dd", "dw", "is", "id", "iw"), tidy)})
            x = lvg.HostGraph(yo, yk, yw, yex)
            print(name, step, "batch", b.num_deletions, b.num_insertions, "tidied", len(tidy[0]), len(tidy[3]),
                  "edges", len(yk))
    np.savez_compressed(os.path.join(OUT, "apply.npz"), **d)


def temporal_fixture(ref) -> None:
    """temporal.npz: a small drifting-community stream (the lines of a SNAP
    temporal file) and the base graph the reference's main.cxx builds from its
    first 90 % (readTemporalOmpW + symmetrizeOmp)."""
    import tempfile

    rows, lines = 3000, 12000
    src, dst, _ = lvg.temporal_drift(rows, 60, lines, seed=5)
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "t.txt")
        lvg.write_temporal(path, src, dst)
        off, key, w, ex = ref.read_temporal(path, rows, int(0.9 * lines))
    np.savez_compressed(os.path.join(OUT, "temporal.npz"), src=src, dst=dst, rows=rows, lines=lines,
                        x_off=off, x_key=key, x_w=w, x_ex=ex)
    print("temporal", rows, lines, "base edges", len(key))


def cases():
    yield "pp2k", lvg.planted_partition(2048, 128, 16, 0.8, 11), 200
    yield "rmat11", lvg.rmat(11, 16, seed=5), 200
    yield "edge", edge_case_graph(), None


def flat_rows(rows):
    r, k, w = [], [], []
    for c, row in enumerate(rows):
        for d in sorted(row):
            r.append(c)
            k.append(d)
            w.append(row[d])
    return np.array(r, np.uint32), np.array(k, np.uint32), np.array(w, np.float64)


def main() -> None:
    lvg_build.build_graphgen()
    # the reference checkout: $LVG_REFERENCE_DIR (the fixtures are generated
    # where the checkout is; the committed .npz files are what the tests read)
    O.build(ref=True)
    ref = O.Reference()
    apply_fixtures(ref)
    temporal_fixture(ref)
    if sys.argv[1:] == ["--only", "apply"]:
        return
    for name, x, nupd in cases():
        b = edge_case_batch(x) if nupd is None else lvg.random_batch(x, nupd, 0.8, seed=7)
        y = lvg.apply_batch(x, b)
        rx, ry = ref.graph(x), ref.graph(y)
        ref.threads(1)
        d = dict(x_off=x.offsets, x_key=x.keys, x_w=x.weights, x_ex=x.exists,
                 y_off=y.offsets, y_key=y.keys, y_w=y.weights, y_ex=y.exists,
                 b_ds=b.del_src, b_dd=b.del_dst, b_dw=b.del_w, b_is=b.ins_src, b_id=b.ins_dst, b_iw=b.ins_w)
        d["x_M"] = rx.edge_weight() / 2
        d["y_M"] = ry.edge_weight() / 2
        d["x_vtot"] = rx.vertex_weights()
        m, vt, ct, info = rx.louvain(0)
        d.update(static_m=m, static_vt=vt, static_ct=ct, static_iter=info["iterations"],
                 static_pass=info["passes"], static_aff=info["affectedVertices"], static_q=rx.modularity(m))
        q, qvt, qct = m, vt, ct
        uvt, uct = ry.update_weights(b, q, qvt, qct)
        d.update(upd_vt=uvt, upd_ct=uct)
        d["df_flags"] = ry.df_mark(b, q)
        dv, dn, dc = ry.ds_mark(b, q, uvt, uct, d["y_M"])
        d.update(ds_vertices=dv, ds_neighbors=dn, ds_communities=dc)
        ren, CN, rows = ry.aggregate(q)
        rr, rk, rw = flat_rows(rows)
        d.update(agg_ren=ren, agg_cn=CN, agg_row=rr, agg_key=rk, agg_w=rw)
        for meth, tag in ((1, "nd"), (2, "ds"), (3, "df")):
            mm, mv, mc, mi = ry.louvain(meth, b, q, qvt, qct)
            d.update({f"{tag}_m": mm, f"{tag}_vt": mv, f"{tag}_ct": mc, f"{tag}_iter": mi["iterations"],
                      f"{tag}_pass": mi["passes"], f"{tag}_aff": mi["affectedVertices"],
                      f"{tag}_q": ry.modularity(mm)})
        ref.threads(8)
        d["static_q_mean8"] = float(np.mean([rx.modularity(rx.louvain(0)[0]) for _ in range(5)]))
        for meth, tag in ((1, "nd"), (2, "ds"), (3, "df")):
            d[f"{tag}_q_mean8"] = float(np.mean([ry.modularity(ry.louvain(meth, b, q, qvt, qct)[0])
                                                 for _ in range(5)]))
        np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **d)
        print(name, "S", x.span, "E", x.num_edges, "batch", b.num_deletions, b.num_insertions,
              "static Q", round(d["static_q"], 6), "passes", d["static_pass"], "CN", CN)

    # Planted partition at the configuration-1 size (131072 vertices): only
    # the reference's modularity, for the tolerance gate at full size.
    x = lvg.planted_partition(131072, 128, 16, 0.8, 42)
    b = lvg.random_batch(x, x.num_edges // 2 // 10000, 0.8, seed=7)
    y = lvg.apply_batch(x, b)
    rx, ry = ref.graph(x), ref.graph(y)
    ref.threads(8)
    runs = [rx.louvain(0) for _ in range(5)]
    qs = [rx.modularity(r[0]) for r in runs]
    m, vt, ct, _ = runs[0]
    dq = {f"{t}_q": [ry.modularity(ry.louvain(meth, b, m, vt, ct)[0]) for _ in range(5)]
          for meth, t in ((1, "nd"), (2, "ds"), (3, "df"))}
    np.savez_compressed(os.path.join(OUT, "pp131k_quality.npz"), static_q=np.array(qs),
                        nd_q=np.array(dq["nd_q"]), ds_q=np.array(dq["ds_q"]), df_q=np.array(dq["df_q"]),
                        prior_m=m, prior_vt=vt, prior_ct=ct, num_updates=b.num_deletions + b.num_insertions)
    print("pp131k static Q mean", np.mean(qs), "df", np.mean(dq["df_q"]))


if __name__ == "__main__":
    main()
