"""bench.py's host-side helpers, without a GPU: the --set-tuning parser, the
launch groups' degree labels, the algorithmic bytes per edge, the clock
summary from either sampler (NVML and nvidia-smi), the peak it divides by and
the config both arms print."""
import argparse
import json
import os

import numpy as np
import pytest

from conftest import ROOT

import bench


def test_parse_tuning_types_and_fields(lvg):
    k = bench.parse_tuning("frontier_colors=1, hub_chunk=16384,frontier_max_fraction=0.25,"
                           "bin_max_degree=0:0:0:8:0:0:0:128:128,")
    assert k == {"frontier_colors": 1, "hub_chunk": 16384, "frontier_max_fraction": 0.25,
                 "bin_max_degree": [0, 0, 0, 8, 0, 0, 0, 128, 128]}
    assert isinstance(k["frontier_max_fraction"], float) and isinstance(k["hub_chunk"], int)
    # every knob the parser yields is a field of lvg_tuning
    assert set(k) <= set(lvg.tuning_default())
    assert bench.parse_tuning("") == {}
    with pytest.raises(ValueError):
        bench.parse_tuning("hub_chunk=big")


def test_group_labels_default_limits():
    labels = [bench.group_label("k", bins, {}) for _, bins in bench.MOVE_GROUPS]
    assert labels == ["degree 1-128 (k)", "degree 129-512 (k)", "degree 513-2048 (k)", "degree 2049-8192 (k)",
                      "degree above 8192 (k)"]


def test_group_labels_tuned_limits():
    # bins 7 and 8 closed at degree 128 hand their degrees to bin 9
    t = {"bin_max_degree": [0, 0, 0, 8, 0, 0, 0, 128, 128, 0, 0, 0]}
    labels = [bench.group_label("k", bins, t) for _, bins in bench.MOVE_GROUPS]
    assert labels == ["degree 1-128 (k)", "no degrees: handed to the next bin (k)", "degree 129-2048 (k)",
                      "degree 2049-8192 (k)", "degree above 8192 (k)"]
    # a wider bin 9 narrows bin 10
    t = {"bin_max_degree": [0] * 9 + [4096, 0, 0]}
    assert bench.group_label("k", [10], t) == "degree 4097-8192 (k)"
    assert bench.group_label("k", [9], t) == "degree 513-4096 (k)"


def test_move_bytes_per_edge(lvg):
    class G:
        def __init__(self, w):
            self.weights = np.asarray(w, np.float32)

    assert bench.move_bytes_per_edge(G([1, 1, 1])) == bench.MOVE_BYTES_PER_EDGE_UNIT
    assert bench.move_bytes_per_edge(G([1, 0.5])) == bench.MOVE_BYTES_PER_EDGE
    assert bench.move_bytes_per_edge(G([])) == bench.MOVE_BYTES_PER_EDGE


class _FakeNvml:
    max_mhz = 2070.0


def test_clock_summary_nvml_reasons():
    c = bench.Clocks(0)
    c.nvml = _FakeNvml()
    c.samples = [(2070.0, set()), (2055.0, {"sw_power_cap"}), (2070.0, None)]
    s = c.summary()
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0 and s["samples"] == 3
    assert s["reasons"] == ["sw_power_cap"]
    assert s["reasons_unread_samples"] == 1


def test_clock_summary_nvml_unread_is_unknown():
    """Samples whose reasons could not be read give reasons None (unknown), not
    an empty list that would read as unthrottled."""
    c = bench.Clocks(0)
    c.nvml = _FakeNvml()
    c.samples = [(2070.0, None), (2070.0, None)]
    assert c.summary()["reasons"] is None
    c.samples = []
    s = c.summary()
    assert s["reasons"] is None and s["samples"] == 0


def test_clock_summary_nvidia_smi_lines():
    c = bench.Clocks(0)
    c.lines = ["2070, 2070, 812.4, Not Active, Not Active, Not Active, Not Active",
               "1980, 2070, 1391.0, Not Active, Not Active, Not Active, Active",
               "2070, 2070, 900.0, Active, Not Active, Not Active, Not Active",
               "[N/A], 2070, 1.0, Not Active, Not Active, Not Active, Not Active",
               "garbage"]
    s = c.summary()
    assert s["samples"] == 3 and s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["hw_slowdown", "sw_power_cap"]
    c.lines = []
    assert c.summary()["reasons"] is None


def test_peak_is_the_measured_copy_bandwidth():
    p, kind = bench.peaks()
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.isfile(path):
        with open(path) as f:
            assert (p, kind) == (float(json.load(f)["hbm_gbs"]), "measured")
    else:
        assert (p, kind) == (6800.0, "fallback")


def test_both_arms_print_one_config():
    a = argparse.Namespace(scale=24, edge_factor=16.0, batch_fraction=1e-4)

    class Y:
        order, num_edges = 16777216, 520800750

    c = bench.bench_config(a, Y, 26038, 26038, 1)
    assert set(c) == {"workload", "vertices", "edges", "batch_updates", "batch_entries", "parallelism", "l2",
                      "prior"}
    assert c["parallelism"] == "replicas x1" and "scale 24" in c["workload"]
    assert c == bench.bench_config(a, Y, 26038, 26038, 1)
