"""Build the GB300 shared library in-tree with nvcc (no cmake).

    python -m bartels_gb300.build          # -> bartels_gb300/lib/libbartels_gpu.so

Each translation unit is compiled for sm_103a in parallel, then linked into one
shared library exposing the C ABI of include/bartels_gpu.h.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIBDIR, "libbartels_gpu.so")
SOURCES = ["elements.cu", "plan.cu", "solver.cu", "amg.cu", "capi.cu", "lpcg.cu", "gemm_tc.cu", "tri.cu", "laws.cu",
           "mex.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags():
    return ARCH + [
        "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
        "-Xcompiler", "-fPIC", "-Xcompiler", "-fopenmp",
        "-I", os.path.join(ROOT, "include"), "-I", CSRC,
    ]


def _compile(src: str) -> str:
    out = os.path.join(OBJ, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), "-c", os.path.join(CSRC, src), "-o", out] + _flags()
    if os.environ.get("BARTELS_PTXAS_VERBOSE"):
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if os.environ.get("BARTELS_PTXAS_VERBOSE"):
        sys.stderr.write(r.stderr)
    return out


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [
        os.path.join(ROOT, "include", h) for h in ("bartels_gpu.h", "bartels_mex.h")]
    return any(os.path.getmtime(p) > t for p in deps)


def build(force: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = [nvcc(), "-shared", "-o", tmp] + objs + ARCH + ["-Xcompiler", "-fopenmp", "-lgomp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
