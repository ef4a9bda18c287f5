#!/usr/bin/env python3
"""Benchmark: dynamic-frontier Louvain edges/s on an R-MAT scale-24 graph.

Workload (the headline configuration): R-MAT scale 24, edge factor 16,
(a,b,c,d) = (0.57,0.19,0.19,0.05), symmetrized and deduplicated (~5.4e8
directed edges), FP32 unit weights, uint32 ids, vertex 0 absent. A step is one
dynamic-frontier Louvain run over one batch of 1e-4 |E| random updates (80 %
insertions of absent uniform pairs, 20 % deletions of uniformly sampled edges)
on the updated graph, from the static Louvain result of the base graph
(deterministic mode, so the prior and the step's work are the same every run).

Arms:
  default              the GPU library. `value` = |E| / per-step device time
                       with graph, batch and prior state resident in HBM
                       (lvg_run_resident, timed by the library's CUDA events);
                       `e2e` = the same through the drop-in call lvg_frontier
                       with host arrays (pinned): batch + prior state uploaded,
                       result downloaded, inside the timed region.
  --impl reference     the CPU implementation of the path on this host's
                       cores, all threads: the reference's own headers
                       compiled here (from its checkout, or from the copy the
                       oracle recipe stages beside the tree), else the
                       oracle's port; same graph, batch and metric, the prior
                       from its own static Louvain (main.cxx:89).

Multi-GPU: the path does not shard (replicas only); under torchrun every rank
runs an independent replica on its own GPU and rank 0 reports the aggregate.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "louvain-communities-openmp-dynamic_gb300")
for _p in (PKG, ROOT):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "DF-Louvain edges/s, HBM GB/s, p99 update latency vs plain GPU at |ΔQ|≤1e-3"
MOVE_BYTES_PER_EDGE = 12   # neighbour id + weight + neighbour's community
MOVE_BYTES_PER_EDGE_UNIT = 8  # the same when every weight is 1: the kernels read no weights
MOVE_BYTES_PER_VERTEX = 25  # offset (8) + degree (4) + community (4) + FP64 vertex weight (8) + flag (1)
HUB_TABLE_BYTES_PER_SLOT = 8  # community (4) + neighbour count (4) of a resident hub table
# the local-moving launches by degree bin: (name, bins); the fused small-bin
# launches time under their first bin
MOVE_GROUPS = [
    ("move_small_kernel<1,6> or move_tile_kernel bins 1-6", [1, 2, 3, 4, 5, 6]),
    ("move_small_kernel<7,8> or move_tile_kernel bins 7-8", [7, 8]),
    ("move_big_kernel, bin 9", [9]),
    ("move_big_kernel, bin 10", [10]),
    ("hub_table_kernel on resident tables; hub_chunk_kernel + hub_merge_kernel for the rest", [11]),
]
BIN_REACH = [0, 4, 8, 16, 32, 64, 128, 256, 512, 2048, 8192]


def group_label(kernels: str, bins, tuning: dict) -> str:
    """A launch group's degree range under the tuning's degree-bin limits."""
    lim = list(tuning.get("bin_max_degree", [0] * 12)) + [0] * 12
    hi = [0] + [lim[b] or BIN_REACH[b] for b in range(1, 11)]
    if bins[0] == 11:
        return f"degree above 8192 ({kernels})"
    lo, top = hi[bins[0] - 1], hi[bins[-1]]
    if top <= lo:
        return f"no degrees: handed to the next bin ({kernels})"
    return f"degree {lo + 1}-{top} ({kernels})"


def parse_tuning(spec: str) -> dict:
    """--set-tuning's knob=value,... as lvg_tuning fields: integers, except
    frontier_max_fraction (a float) and bin_max_degree=a:b:c... (the degree
    bins' limits from bin 0 on)."""
    knobs = {}
    for kv in spec.split(","):
        if not kv.strip():
            continue
        k, v = kv.split("=")
        k = k.strip()
        knobs[k] = (float(v) if k == "frontier_max_fraction" else
                    [int(x) for x in v.split(":")] if k == "bin_max_degree" else int(v))
    return knobs


def move_bytes_per_edge(g) -> int:
    """Algorithmic bytes per scanned edge of the local-moving kernels on host graph g."""
    return MOVE_BYTES_PER_EDGE_UNIT if len(g.weights) and bool(np.all(g.weights == 1.0)) else MOVE_BYTES_PER_EDGE


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--scale", type=int, default=24)
    p.add_argument("--edge-factor", type=float, default=16.0)
    p.add_argument("--batch-fraction", type=float, default=1e-4)
    p.add_argument("--seed", type=int, default=42)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-tune", action="store_true",
                   help="skip lvg_autotune (launch shapes and frontier colour classes) before the timed steps")
    p.add_argument("--cpu-steps", type=int, default=2)
    p.add_argument("--workload", default="df", choices=["df", "sweep", "serving", "temporal", "batched", "link"],
                   help="df: the headline (R-MAT scale 24, one graph); sweep: the same graph, batches of "
                        "1e-7..1e-1 |E|, all four methods; serving: many resident graphs under "
                        "Poisson batch-update arrivals through lvg_server; temporal: a drifting-community "
                        "temporal stream, insertion-only batches, all four methods")
    p.add_argument("--batched-graphs", type=int, default=4096)
    p.add_argument("--batched-loop", type=int, default=512,
                   help="batched: graphs the one-by-one comparator runs (a prefix of the batch)")
    p.add_argument("--drift-vertices", type=int, default=4_000_000)
    p.add_argument("--drift-communities", type=int, default=4000)
    p.add_argument("--stream-batches", type=int, default=1000,
                   help="temporal: consecutive batches of the 1e-5 stream (1e-4: a tenth, 1e-3: a hundredth)")
    p.add_argument("--drift-edges", type=int, default=200_000_000)
    p.add_argument("--graphs", type=int, default=64)
    p.add_argument("--scale-min", type=int, default=18)
    p.add_argument("--scale-max", type=int, default=22)
    p.add_argument("--rate", type=float, default=2000.0, help="serving: offered requests/s")
    p.add_argument("--duration", type=float, default=3.0, help="serving: seconds of arrivals")
    p.add_argument("--size-min", type=int, default=10)
    p.add_argument("--size-max", type=int, default=100000)
    p.add_argument("--workers", type=int, default=16)
    p.add_argument("--budget-gb", type=float, default=120.0)
    p.add_argument("--coalesce", type=int, default=0,
                   help="serving headline: serve a graph's queued requests as one batch of up to this many "
                        "entries (default 0: every request runs alone, with its own result)")
    p.add_argument("--coalesced-mode", type=int, default=1 << 18,
                   help="serving: after the headline, the same arrivals again with coalescing up to this many "
                        "entries, reported as its own labelled mode (0: skip)")
    p.add_argument("--ncu-steps", type=int, default=0,
                   help="profiling mode: set up as usual, then run this many steps between "
                        "cudaProfilerStart/Stop (for ncu --profile-from-start off) and exit")
    p.add_argument("--set-tuning", default="",
                   help="df workload: launch shapes as knob=value,... (lvg_tuning fields) instead of "
                        "running the autotuner, e.g. to profile the shapes a timed run picked")
    p.add_argument("--ncu-method", default="df", choices=["df", "static", "nd", "ds", "apply"],
                   help="profiling mode of the df workload: the call profiled (static: the plain GPU static "
                        "Louvain on the updated graph; nd / ds: naive-dynamic / delta-screening from the prior; "
                        "apply: tidy + apply of the step's batch to a copy of the base graph in HBM)")
    return p.parse_args()


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


class Dist:
    """Barrier and max-over-ranks with torch.distributed (gloo); no-op for one rank."""

    def __init__(self, world: int):
        self.world = world
        self.dist = None
        if world > 1:
            import torch.distributed as dist

            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.dist:
            self.dist.barrier()

    def max(self, x: float) -> float:
        if not self.dist:
            return x
        import torch

        t = torch.tensor([x], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def sum(self, x: float) -> float:
        if not self.dist:
            return x
        import torch

        t = torch.tensor([x], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.dist:
            self.dist.destroy_process_group()


class _NvmlReader:
    """Read-only NVML queries through ctypes (SM clock, its maximum, and the
    active clock-event reasons); None when NVML cannot be loaded."""

    # nvmlClocksEventReasons bits
    BITS = {"sw_power_cap": 0x4, "hw_slowdown": 0x8, "sw_thermal_slowdown": 0x20, "hw_thermal_slowdown": 0x40}

    def __init__(self, index: int):
        import ctypes
        self.c = ctypes
        self.lib = ctypes.CDLL("libnvidia-ml.so.1")
        L, h, u, ull = self.lib, ctypes.c_void_p, ctypes.c_uint, ctypes.c_ulonglong
        L.nvmlInit_v2.argtypes = []
        L.nvmlInit_v2.restype = ctypes.c_int
        L.nvmlShutdown.argtypes = []
        L.nvmlShutdown.restype = ctypes.c_int
        L.nvmlDeviceGetHandleByIndex_v2.argtypes = [u, ctypes.POINTER(h)]
        L.nvmlDeviceGetHandleByIndex_v2.restype = ctypes.c_int
        L.nvmlDeviceGetClockInfo.argtypes = [h, ctypes.c_int, ctypes.POINTER(u)]
        L.nvmlDeviceGetClockInfo.restype = ctypes.c_int
        L.nvmlDeviceGetMaxClockInfo.argtypes = [h, ctypes.c_int, ctypes.POINTER(u)]
        L.nvmlDeviceGetMaxClockInfo.restype = ctypes.c_int
        if L.nvmlInit_v2() != 0:
            raise RuntimeError("nvmlInit failed")
        self.h = h()
        if L.nvmlDeviceGetHandleByIndex_v2(u(index), ctypes.byref(self.h)) != 0:
            raise RuntimeError("no NVML device")
        fn = getattr(L, "nvmlDeviceGetCurrentClocksEventReasons", None)
        self.reasons_fn = fn or L.nvmlDeviceGetCurrentClocksThrottleReasons
        self.reasons_fn.argtypes = [h, ctypes.POINTER(ull)]
        self.reasons_fn.restype = ctypes.c_int
        v = u()
        self.max_mhz = float(v.value) if L.nvmlDeviceGetMaxClockInfo(self.h, 1, ctypes.byref(v)) == 0 else None

    def sample(self):
        """(SM MHz, set of active reasons) — the set is None when the reasons
        could not be read, so an unread sample never looks unthrottled."""
        v, r = self.c.c_uint(), self.c.c_ulonglong()
        if self.lib.nvmlDeviceGetClockInfo(self.h, 1, self.c.byref(v)) != 0:  # 1 = NVML_CLOCK_SM
            return None
        if self.reasons_fn(self.h, self.c.byref(r)) != 0:
            return float(v.value), None
        return float(v.value), {n for n, bit in self.BITS.items() if r.value & bit}

    def close(self):
        self.lib.nvmlShutdown()


class Clocks:
    """Clock sampling during the timed region: in-process NVML reads every
    2 ms (a timed region can be a few milliseconds long), and nvidia-smi at
    100 ms as the fallback where NVML cannot be loaded."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []
        self.nvml = None
        self.samples = []
        self.stop = threading.Event()

    def __enter__(self):
        try:
            self.nvml = _NvmlReader(self.index)
        except Exception:
            self.nvml = None
        if self.nvml:
            self.t = threading.Thread(target=self._poll, daemon=True)
            self.t.start()
            return self
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # the sampler's first line before the timed region starts (a short
            # region would otherwise end before nvidia-smi prints anything)
            t0 = time.time()
            while not self.lines and time.time() - t0 < 3.0:
                time.sleep(0.01)
            self.lines.clear()
        except Exception:
            self.proc = None
        return self

    def _poll(self):
        while not self.stop.is_set():
            x = self.nvml.sample()
            if x:
                self.samples.append(x)
            time.sleep(0.002)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.nvml:
            self.stop.set()
            self.t.join(timeout=2)
            if not self.samples:
                x = self.nvml.sample()
                if x:
                    self.samples.append(x)
            self.nvml.close()
        if self.proc:
            # at least one sample taken from the region's start on
            t0 = time.time()
            while not self.lines and time.time() - t0 < 1.0:
                time.sleep(0.01)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if self.nvml is not None:
            if not self.samples:
                return {"sm_mhz": None, "sm_max_mhz": None, "reasons": None, "samples": 0, "source": "nvml"}
            read = [r for _, r in self.samples if r is not None]
            unread = len(self.samples) - len(read)
            # reasons None: no sample's reasons could be read (unknown, not "none")
            reasons = sorted(set().union(*read)) if read else None
            out = {"sm_mhz": statistics.median(m for m, _ in self.samples), "sm_max_mhz": self.nvml.max_mhz,
                   "reasons": reasons, "samples": len(self.samples), "source": "nvml, 2 ms"}
            if unread:
                out["reasons_unread_samples"] = unread
            return out
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": None, "samples": 0, "source": "nvidia-smi"}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm), "source": "nvidia-smi, 100 ms"}


def make_inputs(lvg, args):
    t = time.time()
    x = lvg.rmat(args.scale, args.edge_factor, 0.57, 0.19, 0.19, seed=args.seed, permute=True)
    nupd = max(1, int(round(args.batch_fraction * x.num_edges / 2)))
    b = lvg.random_batch(x, nupd, 0.8, seed=args.seed + 1)
    y = lvg.apply_batch(x, b)
    return x, b, y, nupd, time.time() - t


def workload_name(args):
    return (f"R-MAT scale {args.scale} (ef {args.edge_factor:g}, a/b/c/d .57/.19/.19/.05), dynamic-frontier "
            f"Louvain per batch of {args.batch_fraction:g}|E| updates (80% ins / 20% del)")


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def traffic_per_launch():
    """DRAM bytes per move launch from the committed ncu summary, if any."""
    try:
        with open(os.path.join(ROOT, "profiles", "move_traffic.json")) as f:
            return json.load(f)
    except Exception:
        return None


def cpu_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


PRIOR = ("deterministic static Louvain on the base graph (16 colour classes): the GPU's in this arm, the "
         "oracle's CPU replay of the same rule in the reference arm — the same membership")


def bench_config(args, y, nupd, batch_entries, world):
    """The workload's config, identical in both arms."""
    return {"workload": workload_name(args), "vertices": y.order, "edges": y.num_edges, "batch_updates": nupd,
            "batch_entries": batch_entries, "parallelism": f"replicas x{world}",
            "l2": "inputs larger than L2 (CSR %.1f GB)" % (y.num_edges * 8 / 1e9), "prior": PRIOR}


def reference_harness():
    """The harness over the reference's own headers (oracle/ref_harness.cxx),
    built from the checkout or from the headers staged next to it, or None
    where neither exists (then the oracle's port stands in)."""
    from oracle import oracle as O

    try:
        O.build(ref=None)
    except Exception:
        return None
    return O.Reference() if O.reference_available() else None


def run_reference(args):
    """The CPU implementation on this host's cores (all threads): the
    reference's own louvainStaticOmp / louvainDynamicFrontierOmp compiled from
    its headers where they are available (kind "reference"), else the oracle's
    port (kind "port"). As main.cxx:89-125 runs it: static Louvain on the base
    graph gives the prior, the batch is tidied and applied in place, then
    dynamic-frontier Louvain. The warm-up and the timed steps are each one call
    with `repeat` repetitions (the reference's LouvainResult::time is the mean
    over them), since every call also allocates span- and edge-sized buffers
    outside its timer."""
    rank, world, _ = dist_info()
    if world > 1 and rank != 0:
        return 0
    import lvg
    import lvg_build
    from oracle import oracle as O

    lvg_build.build_graphgen()
    O.build(ref=False)
    x, b, y, nupd, tgen = make_inputs(lvg, args)
    T = cpu_threads()
    ref = reference_harness()
    orc = O.Oracle()
    extra = {}
    if ref is not None:
        kind = "reference"
        ref.threads(T)
        t0 = time.time()
        R = ref.graph(x)
        t_build = time.time() - t0
        # the prior (untimed, where main.cxx:89 runs static Louvain): the GPU
        # arm's own, deterministic static result, replayed on the CPU by the
        # oracle, so that both arms run DF from the same membership; the
        # reference's own static run is timed beside it (static_reference)
        t0 = time.time()
        m, vt, ct, _ = orc.louvain(x, 0, threads=T, sync=True, colors=16)
        t_prior = time.time() - t0
        q_base = R.modularity(m)
        _, tidy = R.apply_batch(b, csr=False)                # main.cxx:108-109, in place
        tb = lvg.HostBatch(*tidy)
        assert R.size() == y.num_edges
        R.louvain(3, tb, m, vt, ct, opts=O.options(repeat=max(1, args.warmup)))
        md, _, _, inf = R.louvain(3, tb, m, vt, ct, opts=O.options(repeat=args.steps))
        ms = float(inf["time"])
        q_df = R.modularity(md)
        ms_static, q_static = None, None
        if not args.no_cpu_baseline:
            ms2, _, _, sinf = R.louvain(0)
            ms_static, q_static = float(sinf["time"]), R.modularity(ms2)
        # the port beside it, from the same prior (a cross-check of the port)
        pt, pq = [], None
        for _ in range(2):
            pm, _, _, pinf = orc.louvain(y, 3, tb, m, vt, ct, threads=T)
            pt.append(pinf["time"])
            pq = pm
        extra = {"modularity": {"df": q_df, "static_base": q_base, "static_updated": q_static},
                 "static_reference": {"ms": ms_static, "modularity": q_static,
                                      "call": "louvainStaticOmp on the updated graph, one run"},
                 "port_cross_check": {"ms_per_step": float(np.mean(pt)), "modularity": orc.modularity(y, pq),
                                      "call": "the oracle's port (orc_louvain, DF) from the same prior"},
                 "setup_s": {"generate": round(tgen, 1), "reference_graph_build": round(t_build, 1),
                             "prior_replay": round(t_prior, 1)}}
        sample = (f"louvainDynamicFrontierOmp of the reference's own headers (main.sh:54 flags), one call of "
                  f"{args.steps} repetitions after one of {max(1, args.warmup)} (LouvainResult::time, mean over "
                  f"the repetitions), from the deterministic static prior both arms share")
    else:
        kind = "port"
        opts = O.options()
        m, vt, ct, info = orc.louvain(x, 0, threads=T, opts=opts, sync=True, colors=16)  # the shared prior
        times = []
        for i in range(args.warmup + args.steps):
            md, _, _, inf = orc.louvain(y, 3, b, m, vt, ct, threads=T, opts=opts)
            if i >= args.warmup:
                times.append(inf["time"])
        ms = float(np.mean(times))
        extra = {"modularity": {"df": orc.modularity(y, md), "static_base": orc.modularity(x, m)}}
        sample = (f"{args.steps} dynamic-frontier runs of the oracle's port on the full graph (LouvainResult::time: "
                  f"init + mark + passes), from the shared deterministic static prior; the reference's headers were "
                  f"not available")
    value = y.num_edges / (ms / 1e3)
    line = {"metric": METRIC, "value": value, "unit": "edges/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": bench_config(args, y, nupd, b.num_deletions + b.num_insertions, world),
            "cpu_baseline": {"value": value, "unit": "edges/s", "cores": T, "kind": kind, "sample": sample},
            "e2e": {"value": value, "unit": "edges/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    line.update(extra)
    print(json.dumps(line), flush=True)
    return 0


def run_gpu(args):
    rank, world, local = dist_info()
    os.environ.setdefault("CUDA_VISIBLE_DEVICES", os.environ.get("CUDA_VISIBLE_DEVICES", ""))
    dist = Dist(world)
    import lvg
    import lvg_build

    lvg_build.build()
    lvg.set_device(local)  # one replica per GPU, chosen before any handle is created
    x, b, y, nupd, tgen = make_inputs(lvg, args)
    S, E = y.span, y.num_edges

    # prior: static Louvain on the base graph (untimed, as main.cxx:89), in
    # deterministic mode so that every run's DF step starts from the same
    # prior (an asynchronous static result varies run to run, and with it the
    # work a DF step does); the timed DF steps run in the default mode
    X = lvg.Graph(x)
    prior = lvg.louvain_static(X, lvg.LouvainOptions(deterministic=True))
    q_static_base = X.modularity(prior.membership)
    # the batch update itself, in HBM (tidy + apply, lvg_graph_apply_device_batch):
    # the batch and its inverse applied alternately, each a real update of X
    inv = lvg.HostBatch(b.ins_src, b.ins_dst, b.ins_w, b.del_src, b.del_dst, b.del_w)
    apply_ms = []
    for k in range(2 * max(2, args.steps)):
        dbk = lvg.DeviceBatch(X, b if k % 2 == 0 else inv)
        t0 = time.perf_counter()
        X.apply_batch(dbk)
        apply_ms.append((time.perf_counter() - t0) * 1e3)
        dbk.close()
    apply_ms = apply_ms[2:]  # first pair: allocation of the plan buffers
    X.close()
    del X

    Y = lvg.Graph(y)
    st_prior, st_out = lvg.State(Y), lvg.State(Y)
    st_prior.set(prior.membership, prior.vertexWeight, prior.communityWeight)
    db = lvg.DeviceBatch(Y, b)
    o = lvg.LouvainOptions()
    # the library's autotuner picks the launch shapes (and the frontier colour
    # classes, within 1e-3 modularity) on this workload, untimed
    tuning = lvg.get_tuning(Y)
    tune_s = 0.0
    if args.set_tuning:
        tuning = lvg.set_tuning(Y, **parse_tuning(args.set_tuning))
    elif not args.no_tune:
        t0 = time.perf_counter()
        tuning, _ = lvg.autotune(Y, lvg.METHOD_FRONTIER, db, st_prior, o, repeats=9)
        tune_s = time.perf_counter() - t0

    if args.ncu_steps and args.ncu_method == "apply":
        # tidy + apply of the step's batch, on fresh copies of the base graph
        # (a batch applies once): one warm-up copy, then the profiled ones
        X = lvg.Graph(x)
        for k in range(1 + args.ncu_steps):
            C = X.clone()
            dbk = lvg.DeviceBatch(C, b)
            if k:
                lvg.profiler_start()
            C.apply_batch(dbk)
            if k:
                lvg.profiler_stop()
            dbk.close()
            C.close()
        if rank == 0:
            print(json.dumps({"profiled_applies": args.ncu_steps, "batch_entries": b.num_deletions + b.num_insertions}),
                  flush=True)
        dist.close()
        return 0
    if args.ncu_steps:
        meth = {"static": lvg.METHOD_STATIC, "nd": lvg.METHOD_NAIVE, "ds": lvg.METHOD_DELTA,
                "df": lvg.METHOD_FRONTIER}[args.ncu_method]
        # launches one by one (no CUDA graphs: ncu lists the kernels of a
        # graph's conditional node only as the graph), as ncu serialises them anyway
        Y.set_profiling(True)
        lvg.run_resident(Y, meth, db, st_prior, st_out, o)  # warm-up
        lvg.profiler_start()
        for _ in range(args.ncu_steps):
            info = lvg.run_resident(Y, meth, db, st_prior, st_out, o)
        lvg.profiler_stop()
        if rank == 0:
            st = Y.stats()
            print(json.dumps({"profiled_df_steps": args.ncu_steps, "last_ms": info["time"],
                              "kernel_launches_per_step": st["kernel_launches"],
                              "algorithmic_bytes_per_step": move_bytes_per_edge(y) * st["move_edges"] +
                              MOVE_BYTES_PER_VERTEX * st["move_vertices"],
                              "hub_algorithmic_bytes_per_step": move_bytes_per_edge(y) * st["move_bin_edges"][11] +
                              MOVE_BYTES_PER_VERTEX * st["move_bin_vertices"][11]}), flush=True)
        dist.close()
        return 0

    # plain GPU static Louvain on the updated graph (the spec comparator)
    static_times = []
    for _ in range(2):
        info = lvg.run_resident(Y, lvg.METHOD_STATIC, None, None, st_out, o)
        static_times.append(info["time"])
    m_static = st_out.membership()
    q_static = Y.modularity(m_static)

    # warm-up + timed DF steps (inputs resident in HBM; device time by CUDA events)
    for _ in range(args.warmup):
        lvg.run_resident(Y, lvg.METHOD_FRONTIER, db, st_prior, st_out, o)
    step_ms, launches, syncs = [], 0, 0
    dist.barrier()
    with Clocks(local) as clk:
        for _ in range(args.steps):
            info = lvg.run_resident(Y, lvg.METHOD_FRONTIER, db, st_prior, st_out, o)
            step_ms.append(info["time"])
            st = Y.stats()
            launches += st["kernel_launches"]
            syncs += st["host_syncs"]
    dist.barrier()
    # the same steps again with per-launch events around the local-moving kernels (roofline)
    Y.set_profiling(True)
    kms, kedges, kverts, klaunch, kslots = 0.0, 0, 0, 0, 0
    bin_ms, bin_edges, bin_verts = np.zeros(12), np.zeros(12), np.zeros(12)
    for _ in range(args.steps):
        lvg.run_resident(Y, lvg.METHOD_FRONTIER, db, st_prior, st_out, o)
        s = Y.stats()
        kms += s["move_kernel_ms"]
        kedges += s["move_edges"]
        kverts += s["move_vertices"]
        klaunch += s["move_launches"]
        kslots += s["hub_table_slots"]
        bin_ms += np.array(s["move_bin_ms"])
        bin_edges += np.array(s["move_bin_edges"])
        bin_verts += np.array(s["move_bin_vertices"])
    Y.set_profiling(False)
    m_df = st_out.membership()
    q_df = Y.modularity(m_df)
    ms = float(np.mean(step_ms))
    ms_max = dist.max(ms)
    value = world * E / (ms_max / 1e3)

    # e2e: the drop-in call with host (pinned) arrays
    pq = lvg.PinnedArray(S, np.uint32)
    pvt = lvg.PinnedArray(S, np.float64)
    pct = lvg.PinnedArray(S, np.float64)
    pq.array[:] = prior.membership
    pvt.array[:] = prior.vertexWeight
    pct.array[:] = prior.communityWeight
    outs = (lvg.PinnedArray(S, np.uint32), lvg.PinnedArray(S, np.float64), lvg.PinnedArray(S, np.float64))
    ob = tuple(a.array for a in outs)
    for _ in range(max(1, args.warmup)):
        lvg.louvain_dynamic_frontier(Y, b, pq.array, pvt.array, pct.array, o, out_buffers=ob)
    dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        r_e2e = lvg.louvain_dynamic_frontier(Y, b, pq.array, pvt.array, pct.array, o, out_buffers=ob)
    e2e_ms = (time.perf_counter() - t0) * 1e3 / args.steps
    cs = Y.stats()
    e2e_parts = {"upload_ms": cs["call_upload_ms"], "run_ms": cs["call_run_ms"], "download_ms": cs["call_download_ms"],
                 "run_device_ms": float(r_e2e.time), "run_host_syncs": int(cs["host_syncs"])}
    e2e_ms_max = dist.max(e2e_ms)
    h2d = b.num_deletions * 12 + b.num_insertions * 12 + S * (4 + 8 + 8)
    d2h = S * (4 + 8 + 8)

    peak, peak_kind = peaks()
    achieved = None
    bpe = move_bytes_per_edge(y)
    alg_per_step = (bpe * kedges + MOVE_BYTES_PER_VERTEX * kverts + HUB_TABLE_BYTES_PER_SLOT * kslots) / args.steps
    if kms > 0:
        # bytes and time of all local-moving launches of the profiled steps
        achieved = alg_per_step / (kms / args.steps / 1e3) / 1e9
    tr = traffic_per_launch()
    traffic = int(tr["traffic_ratio"] * alg_per_step) if tr and "traffic_ratio" in tr else None
    # the dominant kernel: the launch group of the degree bins with the largest
    # time in the profiled steps (events around each launch). Its algorithmic
    # bytes: per scanned edge and processed vertex as above, plus 8 B per
    # hub-table slot read (community + count) for the vertices above degree 8192
    groups = []
    for kernels, bins in MOVE_GROUPS:
        name = group_label(kernels, bins, tuning)
        gms = sum(bin_ms[k] for k in bins) / args.steps
        galg = sum(bpe * bin_edges[k] + MOVE_BYTES_PER_VERTEX * bin_verts[k] for k in bins) / args.steps
        if 11 in bins:
            galg += HUB_TABLE_BYTES_PER_SLOT * kslots / args.steps
        groups.append((gms, galg, name, bins))
    dom_ms, dom_alg, dom_name, dom_bins = max(groups)
    dom_achieved = dom_alg / (dom_ms / 1e3) / 1e9 if dom_ms > 0 else None
    ratios = (tr or {}).get("group_traffic_ratio", {})
    dom_key = "-".join(str(k) for k in (dom_bins[0], dom_bins[-1]))
    if kslots:
        dom_key += "-tables" if 11 in dom_bins else ""
    dom_traffic = int(ratios[dom_key]["ratio"] * dom_alg) if dom_key in ratios else None
    line = {
        "metric": METRIC, "value": value, "unit": "edges/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": bench_config(args, y, nupd, b.num_deletions + b.num_insertions, world),
        "e2e": {"value": world * E / (e2e_ms_max / 1e3), "unit": "edges/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms_max,
                "call": "lvg_frontier (drop-in for louvainDynamicFrontierOmp), pinned host arrays",
                "last_call_parts": e2e_parts},
        "tuning": dict(tuning, by="--set-tuning" if args.set_tuning else "lvg_autotune" if not args.no_tune else "defaults",
                       seconds=round(tune_s, 2)),
        "gpu_launches": launches,
        "host_syncs_per_step": syncs / args.steps,
        "df_passes_iterations": [info["passes"], info["iterations"]],
        "roofline": {"bound": "hbm", "achieved": dom_achieved, "peak": peak, "unit": "GB/s",
                     "frac": (dom_achieved / peak) if dom_achieved else None,
                     "traffic": dom_traffic,
                     "kernel": dom_name + ": the step's largest kernel time among the local-moving launches",
                     "algorithmic_bytes_per_step": int(dom_alg), "ms_per_step": dom_ms,
                     "traffic_note": ("DRAM bytes of this launch group per step: its ratio to its algorithmic bytes "
                                      "in an ncu capture (" + ratios[dom_key].get("measured_on", "") +
                                      "; profiles/move_traffic.json) times this step's algorithmic bytes")
                                     if dom_traffic else None,
                     "peak_kind": peak_kind,
                     "bound_note": ("latency, not bandwidth: a DF step on a 1e-4 |E| batch processes tens of "
                                    "thousands of vertices, each a chain of dependent gathers; every kernel of the "
                                    "step stays below 7 % of DRAM throughput and 21 % of issue slots in ncu "
                                    "(profiles/move_kernels_rmat22_ncu.md). The hub-scan pair that once dominated "
                                    "the step (0.35 ms, 24 % of the HBM roofline on 58M hub edges) is replaced by "
                                    "resident per-hub community counts (0.04 ms)"),
                     "algorithmic_bytes": f"{bpe} B/scanned edge (neighbour id + its community"
                                          + (", no weight: every weight is 1)" if bpe == 8 else " + weight)")
                                          + f" + {MOVE_BYTES_PER_VERTEX} B/processed vertex"
                                          + f" + {HUB_TABLE_BYTES_PER_SLOT} B/hub-table slot read",
                     "groups_ms_per_step": {name: round(gms, 4) for gms, _, name, _ in groups},
                     "hub_table_slots_per_step": kslots / args.steps,
                     "all_local_moving": {
                         "achieved": achieved, "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                         "algorithmic_bytes_per_step": int(alg_per_step),
                         "kernels": "every degree bin (move_tile/move_small/move_big/hub_table/hub_chunk/hub_merge), "
                                    "durations summed as profiled one after another",
                         "launches_per_step": klaunch / args.steps, "ms_per_step": kms / args.steps,
                         "per_bin_ms_per_step": [round(v / args.steps, 4) for v in bin_ms],
                         "per_bin_edges_per_step": [int(v / args.steps) for v in bin_edges],
                         "per_bin_vertices_per_step": [int(v / args.steps) for v in bin_verts]}},
        "latency_ms": {"p50": float(np.percentile(step_ms, 50)), "p99": float(np.percentile(step_ms, 99))},
        "batch_apply_ms": {"p50": float(np.percentile(apply_ms, 50)), "max": float(np.max(apply_ms)),
                           "call": "lvg_graph_apply_device_batch (tidy + apply in HBM, host wall clock)"},
        "static_gpu": {"ms": float(np.mean(static_times)), "edges_per_s": E / (np.mean(static_times) / 1e3),
                       "modularity": q_static},
        "df_speedup_vs_static_gpu": float(np.mean(static_times)) / ms,
        "modularity": {"df": q_df, "static_updated": q_static, "static_base": q_static_base,
                       "df_minus_static": q_df - q_static},
        "clocks": clk.summary(),
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args, y, b, prior)
        qs = line["cpu_baseline"].pop("static_modularity", None)
        if qs is not None:
            line["static_gpu"]["modularity_cpu_static"] = qs
            line["static_gpu"]["abs_diff_vs_cpu_static"] = abs(q_static - qs)
    if rank == 0:
        print(json.dumps(line), flush=True)
    dist.close()
    return 0


def cpu_baseline(args, y, b, prior):
    """The CPU implementation on the same updated graph, batch and prior (the
    GPU's static result): the reference's own louvainDynamicFrontierOmp where
    its headers are available, else the oracle's port; plus one static run on
    the updated graph, whose modularity the GPU's static result is compared
    with."""
    from oracle import oracle as O

    O.build(ref=False)
    T = cpu_threads()
    q = (prior.membership, prior.vertexWeight, prior.communityWeight)
    ref = reference_harness()
    reps = max(1, args.cpu_steps)
    if ref is not None:
        ref.threads(T)
        R = ref.graph(y)
        m, _, _, inf = R.louvain(3, b, *q, opts=O.options(repeat=reps))
        ms, qd = float(inf["time"]), R.modularity(m)
        sm = R.louvain(0)[0]
        qs = R.modularity(sm)
        kind = "reference"
        sample = (f"louvainDynamicFrontierOmp of the reference's own headers, one call of {reps} repetitions "
                  f"(LouvainResult::time, mean) on the full graph from the GPU's static prior; "
                  f"static_modularity: one louvainStaticOmp run on the updated graph")
    else:
        orc = O.Oracle()
        times = []
        for _ in range(reps):
            m, _, _, inf = orc.louvain(y, 3, b, *q, threads=T)
            times.append(inf["time"])
        ms, qd = float(np.mean(times)), orc.modularity(y, m)
        qs = orc.modularity(y, orc.louvain(y, 0, threads=T)[0])
        kind = "port"
        sample = (f"{reps} dynamic-frontier runs of the oracle's port on the full graph from the GPU's static "
                  f"prior (LouvainResult::time); static_modularity: one static run on the updated graph")
    return {"value": y.num_edges / (ms / 1e3), "unit": "edges/s", "cores": T, "kind": kind, "sample": sample,
            "ms_per_step": ms, "modularity": qd, "static_modularity": qs}


def run_serving(args):
    """Serving: resident R-MAT graphs (scale uniform in [scale-min, scale-max],
    edge factor 16, generated in HBM), Poisson arrivals at `rate`, each request
    a batch of log-uniform [size-min, size-max] undirected updates (20 %
    deletions of edges of the graph, 80 % uniform-pair insertions, both
    directions, drawn as the reference's generators draw them), answered by
    lvg_server (tidy + apply in HBM, then dynamic-frontier Louvain from the
    graph's current state). value = p99 request latency (submit to completion)."""
    rank, world, local = dist_info()
    import lvg
    import lvg_build

    lvg_build.build()
    lvg.set_device(local)
    rng = np.random.default_rng(args.seed)
    budget = int(args.budget_gb * (1 << 30))
    sv = lvg.Server(workers=args.workers, hbm_budget=budget, method=lvg.METHOD_FRONTIER, coalesce=args.coalesce)
    t0 = time.time()
    graphs, ids, refused = [], [], 0
    scales = rng.integers(args.scale_min, args.scale_max + 1, args.graphs)
    for i, sc in enumerate(scales):
        G = None
        try:
            G = lvg.Graph.rmat(int(sc), 16, seed=args.seed + i)
            ids.append(sv.add_graph(G))
            graphs.append(G)
        except lvg.LvgError as e:
            if e.code != lvg.LVG_ENOMEM:
                raise
            refused += 1
            if G is not None:
                G.close()
    t_setup = time.time() - t0
    # launch shapes for the DF requests: the autotuner on the largest graph
    # (a generated batch of 10^4 updates from its static result), copied to all
    t0 = time.time()
    G0 = graphs[int(np.argmax([g.span for g in graphs]))]
    st0 = lvg.State(G0)
    lvg.run_resident(G0, lvg.METHOD_STATIC, None, None, st0, lvg.LouvainOptions())
    db0 = lvg.DeviceBatch.generate(G0, 2000, 8000, seed=args.seed + 999)
    tuning, _ = lvg.autotune(G0, lvg.METHOD_FRONTIER, db0, st0, lvg.LouvainOptions(), repeats=3)
    for g in graphs:
        lvg.set_tuning(g, **tuning)
    db0.close()
    del st0
    t_tune = time.time() - t0

    def payloads_for(n_req, rate, seed):
        """Arrival times, target graphs and host payloads of n_req requests."""
        r = np.random.default_rng(seed)
        at = np.cumsum(r.exponential(1.0 / rate, n_req))
        which = r.integers(0, len(ids), n_req)
        sizes = np.exp(r.uniform(np.log(args.size_min), np.log(args.size_max), n_req)).astype(np.int64)
        pays = [None] * n_req
        for g in range(len(ids)):
            reqs = np.nonzero(which == g)[0]
            if not len(reqs):
                continue
            nd = (sizes[reqs] * 0.2).round().astype(np.int64)
            ni = sizes[reqs] - nd
            db = lvg.DeviceBatch.generate(graphs[g], int(nd.sum()), int(ni.sum()), seed=seed * 1000 + g)
            hb = db.download()
            db.close()
            d0 = i0 = 0
            for q, a, c in zip(reqs, nd, ni):
                # failed deletion draws are dropped by the generator: take what is left in order
                a2 = min(2 * int(a), len(hb.del_src) - d0)
                pays[q] = lvg.HostBatch(hb.del_src[d0:d0 + a2], hb.del_dst[d0:d0 + a2], hb.del_w[d0:d0 + a2],
                                        hb.ins_src[i0:i0 + 2 * c], hb.ins_dst[i0:i0 + 2 * c],
                                        hb.ins_w[i0:i0 + 2 * c])
                d0 += a2
                i0 += 2 * int(c)
        return at, which, pays

    def offered(rate, seed):
        n_req = max(1, int(rate * args.duration))
        at, which, pays = payloads_for(n_req, rate, seed)
        sv.drain()
        sv.stats(reset=True)
        start = time.perf_counter()
        for k in range(n_req):
            while time.perf_counter() - start < at[k]:
                pass
            sv.submit(int(ids[which[k]]), pays[k])
        off_s = time.perf_counter() - start
        sv.drain()
        st = sv.stats()
        st["offered_requests_per_s"] = n_req / off_s
        st["requests"] = n_req
        st["batch_entries"] = int(sum(p.num_deletions + p.num_insertions for p in pays))
        return st

    # warm-up: one small request per graph (capture, workspace)
    for g in ids:
        sv.submit(g, lvg.HostBatch.empty())
    sv.drain()
    sweep = []
    # below the offered rate, and above it (2x, 4x) to find the rate the server sustains
    for i, rate in enumerate(sorted({args.rate / 8, args.rate / 4, args.rate / 2, args.rate * 2, args.rate * 4})):
        st = offered(rate, args.seed + 100 + i)
        sweep.append({"offered_rps": st["offered_requests_per_s"], "achieved_rps": st["requests_per_s"],
                      "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"], "updates_per_s": st["updates_per_s"],
                      "service_ms": {"queue": st["mean_queue_ms"], "apply": st["mean_apply_ms"],
                                     "run": st["mean_run_ms"]}})
    with Clocks(local) as clk:
        st = offered(args.rate, args.seed + 7)
    n_req = st["requests"]
    entries = st["batch_entries"]
    offered_s = n_req / st["offered_requests_per_s"]
    coalesced = None
    if args.coalesced_mode and not args.coalesce:
        # the same kind of arrivals with coalescing: queued requests of a graph
        # share one run (and its result), a throughput mode, labelled as such
        sv.set_coalesce(args.coalesced_mode)
        cst = offered(args.rate, args.seed + 8)
        ovl = offered(args.rate * 4, args.seed + 9)
        sv.set_coalesce(0)
        coalesced = {"mode": f"coalescing up to {args.coalesced_mode} entries: a graph's queued requests run as "
                             "one batch and share its result (a group ends at a conflicting request)",
                     "offered_rps": cst["offered_requests_per_s"], "achieved_rps": cst["requests_per_s"],
                     "p50_ms": cst["p50_ms"], "p99_ms": cst["p99_ms"], "updates_per_s": cst["updates_per_s"],
                     "at_4x_rate": {"offered_rps": ovl["offered_requests_per_s"],
                                    "achieved_rps": ovl["requests_per_s"], "p50_ms": ovl["p50_ms"],
                                    "p99_ms": ovl["p99_ms"], "updates_per_s": ovl["updates_per_s"]}}

    # the plain per-graph loop the server is compared with: requests of the
    # same kind one at a time on one thread (tidy + apply, then DF from the
    # graph's current state, each call synchronous); the states come from the
    # server first (untimed)
    sv.drain()
    nb = 400
    _, lwhich, lpays = payloads_for(nb, args.rate, args.seed + 11)
    o_loop = lvg.LouvainOptions()
    states = []
    for gi, G in enumerate(graphs):
        m, vt, ct = sv.state(ids[gi])
        a, b = lvg.State(G), lvg.State(G)
        a.set(m, vt, ct)
        states.append([a, b])
    t0 = time.perf_counter()
    for k in range(nb):
        gi = int(lwhich[k])
        G = graphs[gi]
        tb = G.apply_batch(lpays[k])
        db = lvg.DeviceBatch(G, tb)
        lvg.run_resident(G, lvg.METHOD_FRONTIER, db, states[gi][0], states[gi][1], o_loop)
        states[gi].reverse()
        db.close()
    loop_s = time.perf_counter() - t0
    loop_entries = int(sum(p.num_deletions + p.num_insertions for p in lpays))
    del states
    line = {
        "metric": "serving p99 update latency (tidy + apply + DF per request)", "value": st["p99_ms"],
        "unit": "ms", "n_gpus": world, "steps": n_req, "warmup": len(ids), "ms_per_step": st["mean_ms"],
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"serving: {len(ids)} resident R-MAT graphs scale {args.scale_min}-{args.scale_max} "
                               f"ef16, Poisson {args.rate:g} req/s for {args.duration:g} s, log-uniform "
                               f"[{args.size_min}, {args.size_max}] updates 80/20, {args.workers} workers, "
                               + (f"coalescing up to {args.coalesce} entries" if args.coalesce
                                  else "every request served alone (no coalescing)"),
                   "graphs": len(ids), "refused_by_admission": refused, "hbm_budget_gb": args.budget_gb,
                   "hbm_reserved_gb": st["hbm_reserved"] / 2**30, "requests": n_req, "batch_entries": entries,
                   "setup_s": t_setup},
        "tuning": dict(tuning, by="lvg_autotune (DF on the largest graph, copied to all)", seconds=round(t_tune, 2)),
        "latency_ms": {"p50": st["p50_ms"], "p99": st["p99_ms"], "mean": st["mean_ms"], "max": st["max_ms"]},
        "service_ms": {"queue": st["mean_queue_ms"], "apply": st["mean_apply_ms"], "run": st["mean_run_ms"]},
        "updates_per_s": st["updates_per_s"], "requests_per_s": st["requests_per_s"],
        "offered_requests_per_s": n_req / offered_s, "completed": st["completed"], "failed": st["failed"],
        "sweep": sweep,
        "one_at_a_time": {"requests": nb, "requests_per_s": nb / loop_s, "batch_entries_per_s": loop_entries / loop_s,
                          "call": "Graph.apply_batch + lvg_run_resident (DF), one request after another"},
        "requests_per_s_vs_one_at_a_time": st["requests_per_s"] / (nb / loop_s),
        "max_sustained_rps": max([st["requests_per_s"]] + [x["achieved_rps"] for x in sweep]),
        "max_sustained_vs_one_at_a_time": max([st["requests_per_s"]] + [x["achieved_rps"] for x in sweep]) /
                                          (nb / loop_s),
        "clocks": clk.summary(),
    }
    if coalesced:
        line["coalesced_mode"] = coalesced
    sv.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def run_temporal(args):
    """Temporal drift: a stream of drift-edges undirected edges over
    drift-vertices vertices in drift-communities log-normal communities
    (sigma 1, 85 % intra), 1 % of the vertices moving every 10M edges; the
    first 90 % form the base graph (main.cxx:159-161), then insertion-only
    batches of 1e-5, 1e-4 and 1e-3 of the stream's lines are tidied and
    applied to a copy of the base (main.cxx:102-109) and static, ND, DS and DF
    Louvain run from the base's static result. value = DF ms at 1e-4.

    Then the stream itself, as main.cxx:101-137 walks it: per batch size,
    --stream-batches consecutive batches (a tenth of that at 1e-4, a
    hundredth at 1e-3) read in order, each tidied and applied in place, with
    ND, DS and DF each starting from its own result on the previous batch;
    static Louvain runs on the final graph, against which the three final
    memberships are compared."""
    rank, world, local = dist_info()
    import lvg
    import lvg_build

    lvg_build.build()
    lvg.set_device(local)
    n, E = args.drift_vertices, args.drift_edges
    t0 = time.time()
    src, dst, _ = lvg.temporal_drift(n, args.drift_communities, E, sigma=1.0, p_in=0.85,
                                     drift_every=10_000_000, drift=0.01, seed=args.seed)
    tgen = time.time() - t0
    base = int(0.9 * E)
    t0 = time.time()
    X = lvg.Graph.from_edges(n + 1, np.concatenate([src[:base], dst[:base]]),
                             np.concatenate([dst[:base], src[:base]]))
    tbuild = time.time() - t0
    o = lvg.LouvainOptions()
    prior = lvg.louvain_static(X, o)
    rows = []
    tuning, tune_s = None, 0.0
    for f in (1e-5, 1e-4, 1e-3):
        k = int(f * E)
        a, b = src[base:base + k], dst[base:base + k]
        ins = lvg.HostBatch(np.zeros(0, np.uint32), np.zeros(0, np.uint32), np.zeros(0, np.float32),
                            np.concatenate([a, b]), np.concatenate([b, a]), np.ones(2 * k, np.float32))
        Y = X.clone()
        t0 = time.perf_counter()
        tb = Y.apply_batch(ins)
        apply_ms = (time.perf_counter() - t0) * 1e3
        if tuning is None:
            # the autotuner picks the frontier methods' launch shapes on the first batch; later
            # copies of the base graph inherit them
            t0 = time.perf_counter()
            st = lvg.State(Y)
            st.set(prior.membership, prior.vertexWeight, prior.communityWeight)
            db = lvg.DeviceBatch(Y, tb)
            tuning, _ = lvg.autotune(Y, lvg.METHOD_FRONTIER, db, st, o, repeats=3)
            lvg.set_tuning(X, **tuning)
            tune_s = time.perf_counter() - t0
        row = {"batch_fraction": f, "lines": k, "tidied_insertions": tb.num_insertions, "apply_ms": apply_ms}
        for name, fn in (("static", None), ("nd", lvg.louvain_naive_dynamic),
                         ("ds", lvg.louvain_dynamic_delta_screening), ("df", lvg.louvain_dynamic_frontier)):
            # the shapes were tuned on DF: the full sweeps keep the default ones
            lvg.set_tuning(Y, **(tuning if name in ("ds", "df") else lvg.tuning_default()))
            ms = []
            for k in range(5):  # two untimed calls first, as in the sweep
                r = lvg.louvain_static(Y, o) if fn is None else fn(Y, tb, prior.membership, prior.vertexWeight,
                                                                    prior.communityWeight, o)
                if k >= 2:
                    ms.append(r.time)
            row[name + "_ms"] = float(np.median(ms))
            row[name + "_q"] = Y.modularity(r.membership)
        row["df_speedup_vs_static"] = row["static_ms"] / row["df_ms"]
        rows.append(row)
        Y.close()
    streams = []
    for f, nb in ((1e-5, args.stream_batches), (1e-4, max(1, args.stream_batches // 10)),
                  (1e-3, max(1, args.stream_batches // 100))):
        k = int(f * E)
        nb = min(nb, (E - base) // max(k, 1))
        Y = X.clone()
        st = {}
        for m in ("nd", "ds", "df"):
            st[m] = [lvg.State(Y), lvg.State(Y)]
            st[m][0].set(prior.membership, prior.vertexWeight, prior.communityWeight)
        db = None
        apply_ms, run_ms = [], {m: [] for m in st}
        pos = base
        for i in range(nb):
            a, b = src[pos:pos + k], dst[pos:pos + k]
            pos += k
            ins = lvg.HostBatch(np.zeros(0, np.uint32), np.zeros(0, np.uint32), np.zeros(0, np.float32),
                                np.concatenate([a, b]), np.concatenate([b, a]), np.ones(2 * k, np.float32))
            t0 = time.perf_counter()
            tb = Y.apply_batch(ins)
            apply_ms.append((time.perf_counter() - t0) * 1e3)
            if db is None:
                db = lvg.DeviceBatch(Y, tb)
            else:
                db.set(tb)
            for m, meth in (("nd", lvg.METHOD_NAIVE), ("ds", lvg.METHOD_DELTA), ("df", lvg.METHOD_FRONTIER)):
                r = lvg.run_resident(Y, meth, db, st[m][0], st[m][1], o)
                run_ms[m].append(r["time"])
                st[m].reverse()  # this batch's result is the next batch's prior
        rs = lvg.louvain_static(Y, o)
        row = {"batch_fraction": f, "batches": nb, "lines_per_batch": k,
               "apply_ms_mean": float(np.mean(apply_ms)), "static_final_ms": rs.time,
               "static_final_q": Y.modularity(rs.membership)}
        for m in st:
            row[m + "_ms_mean"] = float(np.mean(run_ms[m]))
            row[m + "_ms_p99"] = float(np.percentile(run_ms[m], 99))
            row[m + "_final_q"] = Y.modularity(st[m][0].membership())
        row["df_final_minus_static_q"] = row["df_final_q"] - row["static_final_q"]
        streams.append(row)
        for m in st:
            for x in st[m]:
                x.close()
        db.close()
        Y.close()
    mid = rows[1]
    line = {"metric": "temporal drift: DF-Louvain ms per insertion batch", "value": mid["df_ms"], "unit": "ms",
            "n_gpus": world, "steps": 3, "warmup": 2, "ms_per_step": mid["df_ms"], "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"temporal drift: {n} vertices, {args.drift_communities} log-normal communities, "
                                   f"{E} stream edges (90 % base), insertion-only batches 1e-5/1e-4/1e-3",
                       "base_edges": X.size, "generate_s": tgen, "build_graph_s": tbuild},
            "tuning": dict(tuning, by="lvg_autotune (DF, first batch)", seconds=round(tune_s, 2)),
            "batches": rows, "stream": streams}
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def run_sweep(args):
    """Batch-size sweep on the headline graph: R-MAT (scale --scale, ef 16), its
    static result as the prior; for each batch fraction 1e-7 .. 1e-1 of |E|, a
    random batch (80 % uniform-pair insertions, 20 % deletions of existing
    edges, drawn in HBM as the reference's generators draw them) tidied and
    applied to a copy of the base graph, then static, naive-dynamic,
    delta-screening and dynamic-frontier Louvain through the drop-in calls
    (time = LouvainResult::time, median of 3 after 2 untimed calls; modularity of each result). The
    frontier methods' launch shapes come from lvg_autotune at 1e-4 |E|.
    value = DF ms at 1e-4 |E|."""
    rank, world, local = dist_info()
    import lvg
    import lvg_build

    lvg_build.build()
    lvg.set_device(local)
    t0 = time.time()
    G = lvg.Graph.rmat(args.scale, 16, seed=args.seed)
    tgen = time.time() - t0
    E = G.size
    o = lvg.LouvainOptions()
    prior = lvg.louvain_static(G, lvg.LouvainOptions(deterministic=True))

    def updated(f, seed):
        nupd = max(1, int(round(f * E / 2)))
        Y = G.clone()
        db = lvg.DeviceBatch.generate(Y, nupd // 5, nupd - nupd // 5, seed=seed)
        t1 = time.perf_counter()
        Y.apply_batch(db)
        apply_ms = (time.perf_counter() - t1) * 1e3
        return Y, db, nupd, apply_ms

    # launch shapes for the frontier methods, tuned at 1e-4 |E| and inherited by the copies
    t0 = time.perf_counter()
    Y, db, _, _ = updated(1e-4, args.seed + 1)
    st = lvg.State(Y)
    st.set(prior.membership, prior.vertexWeight, prior.communityWeight)
    tuning, _ = lvg.autotune(Y, lvg.METHOD_FRONTIER, db, st, o, repeats=3)
    lvg.set_tuning(G, **tuning)
    del st
    db.close()
    Y.close()
    tune_s = time.perf_counter() - t0
    rows = []
    with Clocks(local) as clk:
        for i, f in enumerate((1e-7, 1e-6, 1e-5, 1e-4, 1e-3, 1e-2, 1e-1)):
            Y, db, nupd, apply_ms = updated(f, args.seed + 10 + i)
            tb = db.download()
            db.close()
            row = {"batch_fraction": f, "updates": nupd, "tidied_entries": tb.num_deletions + tb.num_insertions,
                   "apply_ms": apply_ms}
            for name, fn in (("static", None), ("nd", lvg.louvain_naive_dynamic),
                             ("ds", lvg.louvain_dynamic_delta_screening), ("df", lvg.louvain_dynamic_frontier)):
                # the shapes were tuned on DF: the full sweeps keep the default ones
                lvg.set_tuning(Y, **(tuning if name in ("ds", "df") else lvg.tuning_default()))
                ms = []
                # two untimed calls first: the second captures the phase graph
                # that the timed ones replay (the headline's warm-up)
                for k in range(5):
                    r = lvg.louvain_static(Y, o) if fn is None else fn(Y, tb, prior.membership, prior.vertexWeight,
                                                                        prior.communityWeight, o)
                    if k >= 2:
                        ms.append(r.time)
                row[name + "_ms"] = float(np.median(ms))
                row[name + "_q"] = Y.modularity(r.membership)
            row["df_speedup_vs_static"] = row["static_ms"] / row["df_ms"]
            row["df_minus_static_q"] = row["df_q"] - row["static_q"]
            rows.append(row)
            Y.close()
    mid = [r for r in rows if r["batch_fraction"] == 1e-4][0]
    line = {"metric": "DF-Louvain ms per batch across batch sizes (R-MAT)", "value": mid["df_ms"], "unit": "ms",
            "n_gpus": world, "steps": 3, "warmup": 2, "ms_per_step": mid["df_ms"], "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"R-MAT scale {args.scale} (ef 16, a/b/c/d .57/.19/.19/.05), batches of "
                                   f"1e-7..1e-1 |E| (80 % insertions / 20 % deletions) on copies of the base",
                       "vertices": G.span - 1, "edges": E, "generate_s": tgen},
            "tuning": dict(tuning, by="lvg_autotune (DF at 1e-4 |E|)", seconds=round(tune_s, 2)),
            "batches": rows, "clocks": clk.summary()}
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def batched_specs(n_all: int, seed: int):
    """The batched workload's graphs: |V| log-uniform in [1k, 256k], average
    degree uniform in [8, 32], p_in uniform in [0.6, 0.9] (seeded; the same on
    every rank)."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(1000), np.log(256_000), n_all)).astype(np.int64)
    degs = rng.uniform(8, 32, n_all)
    pins = rng.uniform(0.6, 0.9, n_all)
    return sizes, degs, pins


def rank_share(n_all: int, rank: int, world: int) -> list[int]:
    """The graphs one GPU of `world` clusters: round robin, so the ranks'
    shares are disjoint, cover every graph and differ in size by at most one."""
    return list(range(rank, n_all, world))


def run_batched(args):
    """Batched: planted-partition graphs with |V| log-uniform in [1k, 256k],
    average degree uniform in [8, 32], blocks of 128 (C = |V|/128), p_in
    uniform in [0.6, 0.9], all resident in HBM (generated there). Static
    Louvain on all of them packed back to back as one graph union
    (lvg_static_union: one set of launches per iteration over every graph
    still moving) against lvg_static one graph after another on a prefix, and
    against lvg_static_many (graphs overlapped on the GPU, one stream each).
    value = edges/s of the union run (the union's layout is the input; its
    build from the separate graphs is timed apart). On N GPUs the graphs are
    placed round-robin, one union per GPU, no collective but the timing's
    (total work fixed: strong scaling)."""
    rank, world, local = dist_info()
    import lvg
    import lvg_build

    lvg_build.build()
    lvg.set_device(local)
    dist = Dist(world)
    n_all = args.batched_graphs
    sizes, degs, pins = batched_specs(n_all, args.seed)
    mine = rank_share(n_all, rank, world)  # this GPU's graphs
    t0 = time.time()
    graphs = [lvg.Graph.planted_partition(int(sizes[i]), 128, float(degs[i]), float(pins[i]), args.seed + i)
              for i in mine]
    tgen = time.time() - t0
    n = len(graphs)
    o = lvg.LouvainOptions()
    if args.ncu_steps:  # profiling mode: the union's static runs only
        U = lvg.Graph.union(graphs)
        lvg.louvain_static_union(U, o)
        lvg.profiler_start()
        for _ in range(args.ncu_steps):
            ures = lvg.louvain_static_union(U, o)
        lvg.profiler_stop()
        if rank == 0:
            print(json.dumps({"profiled_union_runs": args.ncu_steps, "graphs": n, "edges": U.size,
                              "last_ms": ures[0].time}), flush=True)
        dist.close()
        return 0
    E = sum(g.size for g in graphs)
    E_all = dist.sum(E)
    o = lvg.LouvainOptions()
    k = min(args.batched_loop, n)
    lvg.louvain_static_many(graphs[:32], o, workers=args.workers, trim=2)  # warm-up
    t0 = time.perf_counter()
    for g in graphs[:k]:
        lvg.louvain_static(g, o)
        g.trim(2)
    loop_s = time.perf_counter() - t0
    Ek = sum(g.size for g in graphs[:k])
    t0 = time.perf_counter()
    res = lvg.louvain_static_many(graphs, o, workers=args.workers, trim=2)
    many_s = time.perf_counter() - t0
    sample = list(range(0, n, max(1, n // 16)))
    qs_many = [graphs[i].modularity(res[i]["membership"]) for i in sample]
    del res
    t0 = time.perf_counter()
    U = lvg.Graph.union(graphs)
    union_build_s = time.perf_counter() - t0
    small = lvg.Graph.union(graphs[:8])
    lvg.louvain_static_union(small, o)  # warm-up (kernel attributes, first launches)
    small.close()
    # launch shapes from the autotuner, tuned on a union of the first 64 graphs
    t0 = time.perf_counter()
    sample_u = lvg.Graph.union(graphs[:64])
    tuning, _ = lvg.autotune(sample_u, lvg.METHOD_STATIC, o=o, repeats=1)
    sample_u.close()
    lvg.set_tuning(U, **tuning)
    tune_s = time.perf_counter() - t0
    dist.barrier()
    with Clocks(local) as clk:
        t0 = time.perf_counter()
        ures = lvg.louvain_static_union(U, o)
        union_s = time.perf_counter() - t0
    union_s = dist.max(union_s)
    ust = U.stats()
    # the same run with the aggregated levels' phases launched the other way
    # (one graph launch per level, or iteration by iteration from the host)
    lg = int(tuning.get("level_graphs", 1))
    lvg.set_tuning(U, level_graphs=1 - lg)
    t0 = time.perf_counter()
    lvg.louvain_static_union(U, o)
    other_s = time.perf_counter() - t0
    ost = U.stats()
    lvg.set_tuning(U, level_graphs=lg)
    run_ms = ures[0].time if ures else 0.0
    qs = [graphs[i].modularity(ures[i].membership) for i in sample]
    line = {"metric": "batched static Louvain edges/s (many graphs)", "value": E_all / union_s, "unit": "edges/s",
            "n_gpus": world, "steps": 1, "warmup": 1, "ms_per_step": union_s * 1e3, "higher_is_better": True,
            "scaling": "strong", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"batched: {n} planted-partition graphs, |V| log-uniform [1k, 256k], degree "
                                   f"U[8, 32], blocks of 128, p_in U[0.6, 0.9], packed back to back as one graph "
                                   f"union; lvg_static_union vs lvg_static one by one",
                       "graphs": n_all, "graphs_per_gpu": n, "vertices": int(sizes.sum()), "edges": int(E_all),
                       "generate_s": tgen,
                       "union_build_s": union_build_s},
            "graphs_per_s": n_all / union_s,
            "tuning": dict(tuning, by="lvg_autotune on a union of 64 of the graphs", seconds=round(tune_s, 2)),
            "union": {"wall_s": union_s, "device_run_ms": run_ms,
                      "local_move_ms": ures[0].localMoveTime if ures else 0.0,
                      "aggregation_ms": ures[0].aggregationTime if ures else 0.0,
                      "first_pass_ms": ures[0].firstPassTime if ures else 0.0,
                      "download_ms": U.stats()["call_download_ms"],
                      "iterations_max": int(max(r.iterations for r in ures)),
                      "passes_max": int(max(r.passes for r in ures)),
                      "host_syncs": int(ust["host_syncs"]), "kernel_launches": int(ust["kernel_launches"]),
                      "level_phase_graphs": int(ust["level_graphs"]),
                      f"wall_s_with_level_graphs_{1 - lg}": other_s,
                      f"host_syncs_with_level_graphs_{1 - lg}": int(ost["host_syncs"])},
            "one_by_one": {"graphs": k, "edges_per_s": Ek / loop_s, "graphs_per_s": k / loop_s},
            "speedup_vs_one_by_one": (E / union_s) / (Ek / loop_s),
            "streams": {"workers": args.workers, "edges_per_s": E / many_s,
                        "speedup_vs_one_by_one": (E / many_s) / (Ek / loop_s),
                        "modularity_sample_mean": float(np.mean(qs_many))},
            "modularity_sample": {"min": float(np.min(qs)), "mean": float(np.mean(qs))},
            "clocks": clk.summary()}
    if rank == 0:
        print(json.dumps(line), flush=True)
    dist.close()
    return 0


def run_link(args):
    """The host link that bounds `e2e`: pinned host <-> device copies of the
    bytes one drop-in call moves each way on R-MAT s24 (the 16.8M-entry prior
    or result: membership u32 + two FP64 weight arrays, 336 MB), as one copy,
    split over 2/4/8 streams, and both directions at once. Best of 5 after a
    warm-up, CUDA events. value = H2D GB/s on one stream."""
    import torch

    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    nbytes = (1 << args.scale) * (4 + 8 + 8)
    h = torch.empty(nbytes, dtype=torch.uint8).pin_memory()
    h2 = torch.empty(nbytes, dtype=torch.uint8).pin_memory()
    d = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    d2 = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    h.fill_(1)
    d2.fill_(2)
    streams = [torch.cuda.Stream() for _ in range(8)]

    def timed(ns, up, down):
        best = 1e30
        for rep in range(6):
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            main = torch.cuda.current_stream()
            e0.record(main)
            chunk = (nbytes + ns - 1) // ns
            for i in range(ns):
                st = streams[i]
                st.wait_event(e0)
                a, b = i * chunk, min(nbytes, (i + 1) * chunk)
                with torch.cuda.stream(st):
                    if up:
                        d[a:b].copy_(h[a:b], non_blocking=True)
                    if down:
                        h2[a:b].copy_(d2[a:b], non_blocking=True)
                main.wait_stream(st)
            e1.record(main)
            e1.synchronize()
            if rep:
                best = min(best, e0.elapsed_time(e1))
        return best

    rows = {}
    for name, up, down in (("h2d", True, False), ("d2h", False, True), ("both", True, True)):
        for ns in (1, 2, 4, 8):
            ms = timed(ns, up, down)
            rows[f"{name}_streams{ns}"] = {"ms": ms, "gb_per_s_each_way": nbytes / ms / 1e6}
    ok = bool((d[:16].cpu() == 1).all() and (h2[:16] == 2).all())
    line = {"metric": "host link copy GB/s (pinned host <-> HBM)", "value": rows["h2d_streams1"]["gb_per_s_each_way"],
            "unit": "GB/s", "n_gpus": 1, "steps": 5, "warmup": 1, "ms_per_step": rows["h2d_streams1"]["ms"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
            "config": {"workload": f"link: {nbytes} B each way (the drop-in call's prior or result at scale "
                                   f"{args.scale})", "bytes": nbytes},
            "copies": rows, "copied_correctly": ok}
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "serving":
        return run_serving(args)
    if args.workload == "temporal":
        return run_temporal(args)
    if args.workload == "batched":
        return run_batched(args)
    if args.workload == "sweep":
        return run_sweep(args)
    if args.workload == "link":
        return run_link(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
