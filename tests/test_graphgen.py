"""Generators (liblvg_graphgen.so): determinism and the reference's input conventions."""
import os
import subprocess
import sys

import numpy as np

from conftest import GOLDEN, PKG


def _valid_symmetric(g):
    S = g.span
    assert g.offsets[0] == 0 and np.all(np.diff(g.offsets.astype(np.int64)) >= 0)
    assert g.exists[0] == 0, "vertex 0 never exists (inc/snap.hxx:133)"
    src = np.repeat(np.arange(S, dtype=np.uint64), np.diff(g.offsets).astype(np.int64))
    dst = g.keys.astype(np.uint64)
    assert np.all(src != dst), "no self-loops"
    key = src * S + dst
    assert np.all(np.diff(key.astype(np.int64)) > 0), "rows sorted and unique"
    rev = np.sort(dst * S + src)
    assert np.array_equal(rev, key), "symmetric"


def test_planted_partition_matches_golden(lvg):
    d = np.load(os.path.join(GOLDEN, "pp2k.npz"))
    g = lvg.planted_partition(2048, 128, 16, 0.8, 11)
    assert np.array_equal(g.offsets, d["x_off"]) and np.array_equal(g.keys, d["x_key"])
    _valid_symmetric(g)


def test_rmat_matches_golden(lvg):
    d = np.load(os.path.join(GOLDEN, "rmat11.npz"))
    g = lvg.rmat(11, 16, seed=5)
    assert np.array_equal(g.offsets, d["x_off"]) and np.array_equal(g.keys, d["x_key"])
    _valid_symmetric(g)


def test_generator_independent_of_thread_count(lvg, tmp_path):
    code = ("import sys; sys.path.insert(0, %r); import lvg, hashlib;"
            "g = lvg.rmat(12, 8, seed=9); b = lvg.random_batch(g, 300, 0.8, 3);"
            "print(hashlib.sha1(g.offsets.tobytes() + g.keys.tobytes() + b.ins_src.tobytes()"
            " + b.del_dst.tobytes()).hexdigest())") % PKG
    outs = []
    for t in ("1", "5"):
        env = dict(os.environ, OMP_NUM_THREADS=t)
        outs.append(subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True,
                                   check=True).stdout.strip())
    assert outs[0] == outs[1]


def test_batch_is_tidy_and_applies(lvg):
    x = lvg.planted_partition(4096, 128, 16, 0.8, 3)
    b = lvg.random_batch(x, 500, 0.8, seed=1)
    assert b.num_insertions == 2 * 400 and b.num_deletions == 2 * 100
    S = x.span
    for src, dst in ((b.del_src, b.del_dst), (b.ins_src, b.ins_dst)):
        k = src.astype(np.int64) * S + dst
        assert np.all(np.diff(k) > 0), "sorted by (src, dst), unique"
        assert np.array_equal(np.sort(dst.astype(np.int64) * S + src), k), "both directions"
    rows = {u: set(x.keys[x.offsets[u]:x.offsets[u + 1]].tolist()) for u in range(S)}
    assert all(int(v) in rows[int(u)] for u, v in zip(b.del_src, b.del_dst)), "deletions exist"
    assert all(int(v) not in rows[int(u)] and u != v for u, v in zip(b.ins_src, b.ins_dst)), "insertions absent"
    y = lvg.apply_batch(x, b)
    assert y.num_edges == x.num_edges - b.num_deletions + b.num_insertions
    _valid_symmetric(y)


def test_empty_batch_apply_is_identity(lvg):
    x = lvg.rmat(9, 8, seed=2)
    y = lvg.apply_batch(x, lvg.HostBatch.empty())
    assert np.array_equal(x.offsets, y.offsets) and np.array_equal(x.keys, y.keys)
