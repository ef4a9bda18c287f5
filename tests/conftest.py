"""Shared fixtures of the test suite.

Markers: ``gpu`` — needs a GB300 (runs the CUDA path through the C-ABI).
Everything else runs on CPU: the oracle against the golden fixtures made by
the reference's own code, the generators, the host logic, and the C-ABI
library's exports.
"""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "louvain-communities-openmp-dynamic_gb300")
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (PKG, ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN_CASES = ["pp2k", "rmat11", "edge"]


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU (runs the CUDA kernels through the C-ABI)")


@pytest.fixture(scope="session")
def lvg():
    import lvg as L
    import lvg_build

    lvg_build.build_graphgen()
    return L


@pytest.fixture(scope="session")
def cuda(lvg):
    """The CUDA library, built for sm_103a and loaded (GPU tests only)."""
    import lvg_build

    lvg_build.build_cuda()
    lvg.load_library()
    return lvg


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle as O

    O.build(ref=False)
    return O.Oracle()


class Golden:
    """One golden case: inputs and the reference's outputs."""

    def __init__(self, name, lvg):
        self.name = name
        self.d = dict(np.load(os.path.join(GOLDEN, f"{name}.npz")))
        d = self.d
        self.x = lvg.HostGraph(d["x_off"], d["x_key"], d["x_w"], d["x_ex"])
        self.y = lvg.HostGraph(d["y_off"], d["y_key"], d["y_w"], d["y_ex"])
        self.b = lvg.HostBatch(d["b_ds"], d["b_dd"], d["b_dw"], d["b_is"], d["b_id"], d["b_iw"])

    def __getitem__(self, k):
        return self.d[k]

    def __contains__(self, k):
        return k in self.d


@pytest.fixture(scope="session", params=GOLDEN_CASES)
def golden(request, lvg):
    return Golden(request.param, lvg)


def rows_sorted(CN, off, keys, w):
    """Aggregated rows as sorted (row, key, weight) arrays."""
    r, k, x = [], [], []
    for c in range(CN):
        o, e = int(off[c]), int(off[c + 1])
        order = np.argsort(keys[o:e], kind="stable")
        r.extend([c] * (e - o))
        k.extend(keys[o:e][order].tolist())
        x.extend(w[o:e][order].tolist())
    return np.array(r, np.uint32), np.array(k, np.uint32), np.array(x, np.float64)
