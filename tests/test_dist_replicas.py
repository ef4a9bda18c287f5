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
