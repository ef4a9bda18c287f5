"""Replica mode of bench.py (one independent replica per GPU): the host-side
rank logic (barrier, max over ranks, whole-job aggregate) on 2 gloo ranks, CPU only."""
import os
import subprocess
import sys

from conftest import ROOT

SCRIPT = r"""
import os, sys, json
sys.path.insert(0, %r)
import bench
rank, world, local = bench.dist_info()
d = bench.Dist(world)
ms = 10.0 + rank            # rank 1 is the slower replica
d.barrier()
ms_max = d.max(ms)
value = world * 1000 / (ms_max / 1e3)
if rank == 0:
    print(json.dumps({"world": world, "ms_max": ms_max, "value": value}))
d.close()
"""


def test_two_rank_max_and_aggregate(tmp_path):
    f = tmp_path / "replica.py"
    f.write_text(SCRIPT % ROOT)
    env = dict(os.environ, MASTER_ADDR="127.0.0.1")
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
                        "--master-addr", "127.0.0.1", "--master-port", "29517", str(f)],
                       capture_output=True, text=True, timeout=240, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    import json
    line = [l for l in r.stdout.splitlines() if l.startswith("{")][-1]
    out = json.loads(line)
    assert out["world"] == 2 and out["ms_max"] == 11.0
    assert abs(out["value"] - 2 * 1000 / 0.011) < 1e-6


BATCHED = r"""
import os, sys, json
sys.path.insert(0, %r)
import numpy as np
import torch.distributed as dist
import bench
rank, world, local = bench.dist_info()
d = bench.Dist(world)
n_all = 37
sizes, degs, pins = bench.batched_specs(n_all, 123)
mine = bench.rank_share(n_all, rank, world)
# the graph specs are the same on every rank (seeded), so a rank's share is a
# function of its index alone
got = [None] * world
dist.all_gather_object(got, {"mine": mine, "sizes": sizes.tolist()})
# the whole job's work, as run_batched sums it over the ranks (strong scaling)
E_all = d.sum(float(sum(int(sizes[i]) * 16 for i in mine)))
t = d.max(1.0 + 0.5 * rank)
if rank == 0:
    print(json.dumps({"shares": [g["mine"] for g in got], "same_specs": all(g["sizes"] == got[0]["sizes"] for g in got),
                      "E_all": E_all, "E_expect": float(sizes.sum() * 16), "t": t}))
d.close()
"""


def test_batched_graphs_split_over_two_ranks(tmp_path):
    """bench.py --workload batched under torchrun: every graph is clustered by
    exactly one rank, the ranks agree on the graphs, and the aggregate sums
    the ranks' edges over the slowest rank's time (gloo, CPU only)."""
    f = tmp_path / "batched_split.py"
    f.write_text(BATCHED % ROOT)
    env = dict(os.environ, MASTER_ADDR="127.0.0.1")
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
                        "--master-addr", "127.0.0.1", "--master-port", "29519", str(f)],
                       capture_output=True, text=True, timeout=240, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    import json
    out = json.loads([l for l in r.stdout.splitlines() if l.startswith("{")][-1])
    a, b = (set(x) for x in out["shares"])
    assert not (a & b) and (a | b) == set(range(37)) and abs(len(a) - len(b)) <= 1
    assert out["same_specs"]
    assert out["E_all"] == out["E_expect"] and out["t"] == 1.5
