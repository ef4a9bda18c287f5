"""The reference's input path and experiment driver: SNAP temporal streams
(inc/snap.hxx), the base graph main.cxx builds from them, main.cxx's flow
and log lines (louvain_gb300_experiment) and process.js's CSV (lvg_log.py).

CPU: the reader + lvgg_csr_from_edges against the graph the reference's own
readTemporalOmpW + symmetrizeOmp built from the same lines
(tests/golden/temporal.npz); the log-line format and its CSV. GPU: the driver
end to end on that stream.
"""
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN


def _fixture():
    return np.load(os.path.join(GOLDEN, "temporal.npz"))


def _write(lvg, d, path):
    lvg.write_temporal(path, d["src"], d["dst"])


def test_base_graph_equals_reference(lvg, tmp_path):
    d = _fixture()
    path = str(tmp_path / "t.txt")
    _write(lvg, d, path)
    rows, lines = int(d["rows"]), int(d["lines"])
    r = lvg.TemporalReader(path)
    s, t, w = r.read(int(0.9 * lines), symmetric=True)
    x = lvg.csr_from_edges(rows, s, t, w)
    assert np.array_equal(x.offsets, d["x_off"])
    assert np.array_equal(x.keys, d["x_key"])
    assert np.array_equal(x.weights, d["x_w"])
    assert np.array_equal(x.exists, d["x_ex"])
    # the stream goes on where the base stopped
    s2, t2, _ = r.read(10, symmetric=False)
    k = int(0.9 * lines)
    assert np.array_equal(s2, d["src"][k:k + 10]) and np.array_equal(t2, d["dst"][k:k + 10])
    r.close()


def test_reader_emits_both_directions_in_order(lvg, tmp_path):
    path = str(tmp_path / "s.txt")
    src = np.array([3, 1, 2, 2], np.uint32)
    dst = np.array([1, 2, 3, 2], np.uint32)
    lvg.write_temporal(path, src, dst)
    s, t, w = lvg.TemporalReader(path).read(100)
    assert s.tolist() == [3, 1, 1, 2, 2, 3, 2, 2] and t.tolist() == [1, 3, 2, 1, 3, 2, 2, 2]
    assert np.all(w == 1)
    x = lvg.csr_from_edges(4, s, t, w)
    assert x.exists.tolist() == [0, 1, 1, 1, 1]  # vertices 1..rows
    assert x.keys[x.offsets[2]:x.offsets[3]].tolist() == [1, 2, 3]  # self-loop kept once


def test_drift_stream_shape(lvg):
    src, dst, w = lvg.temporal_drift(5000, 50, 20000, seed=9)
    assert len(src) == 20000 and src.min() >= 1 and src.max() <= 5000 and dst.max() <= 5000
    a = lvg.temporal_drift(5000, 50, 20000, seed=9)
    assert np.array_equal(a[0], src) and np.array_equal(a[1], dst)
    assert not np.array_equal(lvg.temporal_drift(5000, 50, 20000, seed=10)[0], src)


def test_log_lines_and_csv(tmp_path):
    import lvg_log

    r = dict(time=12.34, markingTime=0.5, initializationTime=0.25, firstPassTime=10.0, localMoveTime=8.0,
             aggregationTime=3.5, affectedVertices=1234, iterations=7, passes=3)
    ln = lvg_log.result_line(r, "louvainDynamicFrontierOmp", 152, 0.7901234567, 0.0, 1e-4)
    assert ln == ("{-0.000e+00/+1.000e-04 batchf, 152 threads} -> {0000012.3ms, 0000000.5ms mark, 0000000.2ms init, "
                  "0000010.0ms firstpass, 0000008.0ms locmove, 0000003.5ms aggr, 1.234e+03 aff, 0007 iters, "
                  "003 passes, 0.790123457 modularity} louvainDynamicFrontierOmp")
    log = tmp_path / "run.log"
    log.write_text("2026-01-02 03:04:05 OMP_NUM_THREADS=152\n"
                   "2026-01-02 03:04:05 Loading graph /data/sx-mathoverflow.txt ...\n"
                   "2026-01-02 03:04:06 order: 24818 size: 187986 [directed] {} (90%)\n"
                   + ln.replace("DynamicFrontier", "StaticOriginal").replace("+1.000e-04", "+0.000e+00") + "\n"
                   "2026-01-02 03:04:07 order: 24818 size: 188000 [directed] {} (insertions=14)\n" + ln + "\n")
    rows = lvg_log.rows_of(lvg_log.read_log(str(log)))
    assert len(rows) == 2
    assert rows[0]["graph"] == "sx-mathoverflow" and rows[0]["batch_index"] == -1
    assert rows[1]["batch_index"] == 0 and rows[1]["technique"] == "louvainDynamicFrontierOmp"  # as process.js counts
    assert rows[1]["modularity"] == 0.790123457 and rows[1]["num_threads"] == 152
    out = tmp_path / "out.csv"
    lvg_log.write_csv(str(out), rows)
    head = out.read_text().splitlines()[0].split(",")
    assert head[:3] == ["omp_num_threads", "graph", "order"] and head[-1] == "technique"


def test_experiment_driver_rejects_bad_arguments(lvg, tmp_path):
    """The experiment driver's command line (main.cxx's: file, rows, size,
    unused, batch fraction; or --drift) fails before any device work: usage
    and status 2 for too few arguments, status 1 naming the failing call for
    an unreadable stream or a --drift line without its batch fraction."""
    import lvg_build

    lvg_build.build_cuda()
    exe = lvg_build.build_experiment()
    r = subprocess.run([exe, "a", "1", "2"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2 and "usage:" in r.stderr and "--drift" in r.stderr
    r = subprocess.run([exe, str(tmp_path / "missing.txt"), "10", "100", "0", "0.01"], capture_output=True,
                       text=True, timeout=60)
    assert r.returncode == 1 and r.stderr.strip() == "lvgg_temporal_open: cannot open the file", r.stderr
    r = subprocess.run([exe, "--drift", "100", "4", "1000", "7"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and r.stderr.strip() == "--drift: missing batchFraction", r.stderr


@pytest.mark.gpu
def test_device_graph_from_edges_equals_reference(cuda, tmp_path):
    d = _fixture()
    path = str(tmp_path / "t.txt")
    _write(cuda, d, path)
    rows, lines = int(d["rows"]), int(d["lines"])
    s, t, w = cuda.TemporalReader(path).read(int(0.9 * lines), symmetric=True)
    G = cuda.Graph.from_edges(rows + 1, s, t, w)
    h = G.download()
    assert np.array_equal(h.offsets, d["x_off"]) and np.array_equal(h.keys, d["x_key"])
    assert np.array_equal(h.weights, d["x_w"]) and np.array_equal(h.exists, d["x_ex"])
    assert G.order == int(d["x_ex"].sum())
    C = G.clone()  # an independent copy
    k = int(np.nonzero(s != t)[0][0])  # an edge that is not a self-loop, both directions
    ds, dd = np.array([s[k], t[k]], np.uint32), np.array([t[k], s[k]], np.uint32)
    C.apply_batch(cuda.HostBatch(ds, dd, np.ones(2, np.float32), np.zeros(0, np.uint32), np.zeros(0, np.uint32),
                                 np.zeros(0, np.float32)))
    assert C.size == G.size - 2 and np.array_equal(G.download().keys, h.keys)


@pytest.mark.gpu
def test_experiment_driver_end_to_end(cuda, tmp_path):
    import lvg_build
    import lvg_log

    lvg_build.build_experiment()
    d = _fixture()
    path = str(tmp_path / "stream.txt")
    _write(cuda, d, path)
    env = dict(os.environ, BATCH_LENGTH="2", REPEAT_METHOD="1")
    out = subprocess.run([cuda.experiment_path(), path, str(int(d["rows"])), str(int(d["lines"])), "0", "0.01"],
                         capture_output=True, text=True, env=env, timeout=300)
    assert out.returncode == 0, out.stderr
    log = tmp_path / "run.log"
    log.write_text(out.stdout)
    rows = lvg_log.rows_of(lvg_log.read_log(str(log)))
    techs = [r["technique"] for r in rows]
    assert techs == ["louvainStaticOmpOriginal"] + 2 * ["louvainStaticOmp", "louvainNaiveDynamicOmp",
                                                         "louvainDynamicDeltaScreeningOmp",
                                                         "louvainDynamicFrontierOmp"]
    base = int(np.sum(d["x_ex"]))
    assert all(r["order"] >= base for r in rows)
    q_static = [r["modularity"] for r in rows if r["technique"] == "louvainStaticOmp"]
    q_df = [r["modularity"] for r in rows if r["technique"] == "louvainDynamicFrontierOmp"]
    assert all(abs(a - b) < 0.02 for a, b in zip(q_static, q_df)), (q_static, q_df)
    assert all(r["batch_insertions_fraction"] == 0.01 for r in rows[1:])


def test_csr_from_edges_keeps_the_last_weight(lvg):
    """lvgg_csr_from_edges against a plain model: rows sorted by neighbour,
    a repeated edge keeps its last weight, vertices 1..rows and every
    endpoint present; an id above rows is refused."""
    rng = np.random.default_rng(17)
    rows, n = 300, 5000
    src = rng.integers(1, rows + 1, n).astype(np.uint32)
    dst = rng.integers(1, rows + 1, n).astype(np.uint32)
    src[:500], dst[:500] = src[500:1000], dst[500:1000]  # repeats, with other weights
    w = rng.integers(1, 100, n).astype(np.float32)
    x = lvg.csr_from_edges(rows, src, dst, w)
    model = [dict() for _ in range(rows + 1)]
    for u, v, a in zip(src.tolist(), dst.tolist(), w.tolist()):
        model[u][v] = a  # later entries overwrite earlier ones
    assert x.span == rows + 1 and x.exists.tolist() == [0] + [1] * rows
    for u in range(rows + 1):
        o, e = int(x.offsets[u]), int(x.offsets[u + 1])
        assert x.keys[o:e].tolist() == sorted(model[u]), u
        assert x.weights[o:e].tolist() == [model[u][v] for v in sorted(model[u])], u
    with pytest.raises(lvg.LvgError):
        lvg.csr_from_edges(rows, np.array([rows + 1], np.uint32), np.array([1], np.uint32))
