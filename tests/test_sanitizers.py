"""Host code under AddressSanitizer + UndefinedBehaviorSanitizer (leaks
included): the MATLAB facade against a stand-in C ABI, the sim:: plan cache,
the CPU oracle and baseline through every entry point, and the kernels'
element math (devmath.cuh) compiled for the host over hard deformations. Any out-of-bounds
access, use after free, leak or undefined arithmetic fails the run. Skipped
where the compiler has no sanitizer runtime."""
import os
import subprocess

import pytest

from conftest import ROOT

SAN = ["-fsanitize=address,undefined", "-fno-omit-frame-pointer", "-g", "-O1", "-std=c++17"]
ENV = dict(os.environ, ASAN_OPTIONS="detect_leaks=1", UBSAN_OPTIONS="halt_on_error=1:print_stacktrace=1",
           OMP_NUM_THREADS="2")

PROGRAMS = {
    "mex_facade": (["tests/mex_fake_abi.cpp", "bartels_gb300/csrc/mex.cpp"], ["-Iinclude"], "mex facade ok"),
    "plan_cache": (["tests/sim_plan_cache_test.cpp"], ["-Iinclude"], "plan cache ok"),
    "oracle": (["tests/oracle_sanitize_driver.cpp", "oracle/oracle_capi.cpp", "oracle/oracle_baseline.cpp"],
               ["-Ioracle", "-fopenmp"], "oracle sanitize ok"),
    "devmath": (["tests/devmath_sanitize_driver.cpp", "tests/devmath_harness.cpp"], ["-Ibartels_gb300/csrc"],
                "devmath sanitize ok"),
}


@pytest.mark.parametrize("name", sorted(PROGRAMS))
def test_host_code_is_sanitizer_clean(name):
    srcs, flags, marker = PROGRAMS[name]
    out_dir = os.path.join(ROOT, "tests", "_build")
    os.makedirs(out_dir, exist_ok=True)
    exe = os.path.join(out_dir, f"san_{name}")
    r = subprocess.run(["g++"] + SAN + [os.path.join(ROOT, s) for s in srcs] +
                       [f.replace("-I", "-I" + ROOT + "/") if f.startswith("-I") else f for f in flags] + ["-o", exe],
                       capture_output=True, text=True)
    if r.returncode != 0 and ("asan" in r.stderr or "ubsan" in r.stderr):
        pytest.skip("no sanitizer runtime: " + r.stderr.strip().splitlines()[-1])
    assert r.returncode == 0, r.stderr
    run = subprocess.run([exe], capture_output=True, text=True, timeout=300, env=ENV)
    assert run.returncode == 0 and marker in run.stdout, run.stderr[-4000:]
