"""bench.py's host logic without a GPU: the clock record that decides whether
a run is kept (median SM clock under load, maximum clock, throttle reasons
seen during the timed region), its handling of malformed samples and of a
machine without nvidia-smi, and the PCG-count file the CPU baseline scales
by."""
import argparse
import json
import os

import bench


def test_clock_summary_median_max_and_reasons():
    c = bench.Clocks(0)
    c.lines = [
        "2070, 2070, 812.3, Not Active, Not Active, Not Active, Not Active",
        "1965, 2070, 1398.0, Not Active, Not Active, Not Active, Active",
        "2070, 2070, 1401.7, Not Active, Not Active, Not Active, Active",
        "[N/A], 2070, 10.0, Not Active, Not Active, Not Active, Not Active",   # unreadable: skipped
        "2070, 2070",                                                           # truncated: skipped
    ]
    s = c.summary()
    assert s == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"], "samples": 3}


def test_clock_summary_flags_thermal_and_hardware_slowdown():
    c = bench.Clocks(0)
    c.lines = ["1400, 2070, 900, Active, Not Active, Active, Not Active"]
    assert c.summary()["reasons"] == ["hw_slowdown", "sw_thermal_slowdown"]


def test_clocks_without_nvidia_smi_record_nothing(monkeypatch):
    monkeypatch.setenv("PATH", "/nonexistent")
    with bench.Clocks(0) as c:
        pass
    assert c.summary() == {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}


def test_newton_counts_file_matches_the_default_workload():
    with open(os.path.join(bench.ROOT, "profiles", "newton_counts.json")) as f:
        c = json.load(f)
    args = argparse.Namespace(n=96, model="neohookean")
    counts = bench.load_counts(args)
    assert counts["pcg_per_newton"] == c["pcg_per_newton"] > 0
    other = bench.load_counts(argparse.Namespace(n=12, model="stvk"))
    assert other["source"] == "default"
