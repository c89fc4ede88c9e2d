"""bench.py's host logic without a GPU: the clock record that decides whether
a run is kept (median SM clock under load, maximum clock, throttle reasons
seen during the timed region), its handling of malformed samples and of a
machine without nvidia-smi, and the PCG-count file the CPU baseline scales
by."""
import argparse
import json
import os
import time

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


def test_reference_arm_times_whole_newton_iterations():
    """--impl reference on a small cube: every timed step is a whole measured
    Newton iteration (no sampled or scaled piece), time steps advance when
    they converge, and the record's time per step adds up to the steps timed."""
    args = argparse.Namespace(n=3, model="neohookean", no_psd=False, steps=12, warmup=2)
    t0 = time.perf_counter()
    out = bench.run_reference(args)
    wall = time.perf_counter() - t0
    assert out["impl"] == "reference" and out["unit"] == bench.UNIT
    assert len(out["seconds_per_step"]) == 12
    assert abs(out["ms_per_step"] * 12 - 1e3 * sum(out["seconds_per_step"])) < 1e-6
    assert out["ms_per_step"] * 12 <= 1e3 * wall
    assert out["cpu_baseline"]["estimated"] is False
    assert out["pcg_iters_per_newton"] > 0
    assert out["time_steps_completed"] >= 1  # 12 Newton iterations finish at least one time step
    assert out["e2e"]["h2d_bytes_per_step"] == 0
