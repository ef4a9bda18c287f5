"""The reference's CPU-runnable case at full size: a planted partition of
131072 vertices in 1024 communities of 128, average degree 16, 80 % of the
edges inside a community; one update batch of 1e-4 |E| (80 % insertions,
20 % deletions).

Deterministic mode: static and dynamic-frontier Louvain on the GPU equal the
CPU replay of the same rule bit for bit. Asynchronous mode (the reference's
semantics): the GPU's modularity is within 0.005 of the mean of 5 runs of the
oracle's OpenMP port, for static and for all three dynamic methods; and, on
the graph and batch of tests/golden/pp131k_quality.npz, within 0.005 of the
mean of 5 runs of the reference's own code (the fixture), the dynamic methods
starting from the reference's own static result.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def case(lvg):
    x = lvg.planted_partition(131072, 128, 16, 0.8, seed=2024)
    b = lvg.random_batch(x, int(round(1e-4 * x.num_edges / 2)), 0.8, seed=2025)
    return x, b, lvg.apply_batch(x, b)


def test_deterministic_static_and_frontier_equal_cpu_replay(cuda, orc, case):
    x, b, y = case
    o = cuda.LouvainOptions(deterministic=True)
    r0 = cuda.louvain_static(cuda.Graph(x), o)
    m, vt, ct, info = orc.louvain(x, 0, threads=8, sync=True)
    assert np.array_equal(r0.membership, m) and np.array_equal(r0.communityWeight, ct)
    assert (r0.iterations, r0.passes) == (info["iterations"], info["passes"])
    r = cuda.louvain_dynamic_frontier(cuda.Graph(y), b, r0.membership, r0.vertexWeight, r0.communityWeight, o)
    m, vt, ct, info = orc.louvain(y, 3, b, r0.membership, r0.vertexWeight, r0.communityWeight, threads=8, sync=True)
    assert np.array_equal(r.membership, m) and np.array_equal(r.communityWeight, ct)
    assert (r.iterations, r.passes, r.affectedVertices) == (info["iterations"], info["passes"],
                                                            info["affectedVertices"])


def test_async_modularity_within_tolerance_of_reference_mean(cuda, orc, case):
    x, b, y = case
    tol = 0.005
    qs = [orc.modularity(x, orc.louvain(x, 0, threads=8)[0]) for _ in range(5)]
    r0 = cuda.louvain_static(cuda.Graph(x))
    assert abs(orc.modularity(x, r0.membership) - np.mean(qs)) <= tol, (orc.modularity(x, r0.membership), qs)
    # the dynamic methods from the same (GPU) prior on the updated graph
    prior = (r0.membership, r0.vertexWeight, r0.communityWeight)
    Y = cuda.Graph(y)
    for method, fn in ((1, cuda.louvain_naive_dynamic), (2, cuda.louvain_dynamic_delta_screening),
                       (3, cuda.louvain_dynamic_frontier)):
        ref = [orc.modularity(y, orc.louvain(y, method, b, *prior, threads=8)[0]) for _ in range(5)]
        q = orc.modularity(y, fn(Y, b, *prior).membership)
        assert abs(q - np.mean(ref)) <= tol, (method, q, ref)


def test_async_modularity_within_tolerance_of_reference_fixture(cuda):
    """Against the reference itself: its 5-run modularities on this graph and
    batch (seeded as in tests/golden/make_golden.py), the dynamic methods from
    its own static result, stored in the fixture."""
    d = np.load(os.path.join(GOLDEN, "pp131k_quality.npz"))
    x = cuda.planted_partition(131072, 128, 16, 0.8, 42)
    b = cuda.random_batch(x, x.num_edges // 2 // 10000, 0.8, seed=7)
    assert b.num_deletions + b.num_insertions == int(d["num_updates"])
    y = cuda.apply_batch(x, b)
    tol = 0.005
    X, Y = cuda.Graph(x), cuda.Graph(y)
    q = X.modularity(cuda.louvain_static(X).membership)
    assert abs(q - d["static_q"].mean()) <= tol, (q, d["static_q"])
    prior = (d["prior_m"], d["prior_vt"], d["prior_ct"])
    for tag, fn in (("nd", cuda.louvain_naive_dynamic), ("ds", cuda.louvain_dynamic_delta_screening),
                    ("df", cuda.louvain_dynamic_frontier)):
        q = Y.modularity(fn(Y, b, *prior).membership)
        assert abs(q - d[f"{tag}_q"].mean()) <= tol, (tag, q, d[f"{tag}_q"])
