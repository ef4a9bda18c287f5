"""`bench.py --impl reference` on CPU at a small scale: the reference arm's
one JSON line keeps the contract the GPU arm's line keeps (metric, unit,
direction, config keys), describes its CPU run (cpu_baseline) and declares no
host-device copies; under a multi-rank launch only rank 0 runs and prints."""
import json
import os
import subprocess
import sys

from conftest import ROOT

import bench


def _run(extra_env=None, gpus=1):
    env = dict(os.environ, **(extra_env or {}))
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--scale", "11",
                        "--steps", "2", "--warmup", "3", "--gpus", str(gpus)],
                       capture_output=True, text=True, env=env, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    return [ln for ln in r.stdout.splitlines() if ln.startswith("{")]


def test_reference_arm_line(lvg):
    lines = _run()
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC and d["unit"] == "edges/s"
    assert d["higher_is_better"] is True and d["steps"] == 2 and d["warmup"] == 3 and d["n_gpus"] == 1
    assert d["value"] > 0 and d["ms_per_step"] > 0
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["unit"] == d["unit"] and cb["kind"] in ("reference", "port")
    assert cb["cores"] >= 1 and cb["sample"]
    # the same config keys as the GPU arm's line (bench_config builds both)
    assert set(d["config"]) == {"workload", "vertices", "edges", "batch_updates", "batch_entries", "parallelism",
                                "l2", "prior"}
    assert "scale 11" in d["config"]["workload"]
    # the modularity the step reaches, from the shared deterministic prior
    assert abs(d["modularity"]["df"] - d["modularity"]["static_base"]) < 0.01


def test_reference_arm_runs_on_rank_zero_only(lvg):
    env = {"WORLD_SIZE": "2", "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": "29555"}
    assert _run(dict(env, RANK="1", LOCAL_RANK="1"), gpus=2) == []
    lines = _run(dict(env, RANK="0", LOCAL_RANK="0"), gpus=2)
    assert len(lines) == 1 and json.loads(lines[0])["n_gpus"] == 2
