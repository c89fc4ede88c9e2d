"""C ABI checks that need no GPU: the library loads, exports every function
declared in include/*.h, and its host-only entry points (integer
bookkeeping, the host line search) agree with the oracle. Also the Kuhn cube
generator's counts against the assembled pattern."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT, gpu_available

import bartels_gb300 as bg
from bartels_gb300 import _lib
from bartels_gb300.meshes import cube_counts, kuhn_cube


def declared_functions():
    inc = os.path.join(ROOT, "include")
    text = "".join(open(os.path.join(inc, h)).read() for h in sorted(os.listdir(inc)) if h.endswith(".h"))
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(bartels_[A-Za-z0-9_]+)\s*\(", text)) - {"bartels_objective_fn"})


def declared_arity():
    """Parameter count of every bartels_* function declared in include/*.h."""
    inc = os.path.join(ROOT, "include")
    text = "".join(open(os.path.join(inc, h)).read() for h in sorted(os.listdir(inc)) if h.endswith(".h"))
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    out = {}
    for m in re.finditer(r"\b(bartels_[A-Za-z0-9_]+)\s*\(", text):
        name, i, depth = m.group(1), m.end(), 1
        j = i
        while depth and j < len(text):
            depth += {"(": 1, ")": -1}.get(text[j], 0)
            j += 1
        params = text[i:j - 1].strip()
        if not params or params == "void":
            n = 0
        else:
            n, d = 1, 0
            for ch in params:
                d += {"(": 1, ")": -1}.get(ch, 0)
                n += ch == "," and d == 0
        if text[j:j + 1].strip() in (";", "") or text[j:].lstrip().startswith(";"):
            out.setdefault(name, n)
    return out


def test_bindings_match_header_arity():
    """Every ctypes binding passes as many arguments as the header declares."""
    ar = declared_arity()
    wrong = [(name, len(args), ar[name]) for name, _, args in _lib.SIGNATURES if name in ar and len(args) != ar[name]]
    assert not wrong, wrong


def test_library_loads_and_exports_header():
    L = bg.lib()
    names = declared_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    # the ctypes signature table covers what the Python mirror calls
    for name, _, _ in _lib.SIGNATURES:
        assert name in names


def test_status_strings():
    L = bg.lib()
    assert L.bartels_status_string(0) == b"ok"
    assert L.bartels_status_string(_lib.E_NOT_CONVERGED) == b"not converged"


def test_context_without_gpu_is_an_error():
    if gpu_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    assert bg.lib().bartels_ctx_create(0, C.byref(h)) == _lib.E_NO_DEVICE
    with pytest.raises(bg.BartelsError):
        bg.Context(0)


def test_fixed_point_constraint_matrix_matches_oracle(oracle):
    rng = np.random.default_rng(0)
    for nV in (1, 5, 40):
        fixed = np.sort(rng.choice(nV, size=rng.integers(0, nV), replace=False)).astype(np.int32)
        V = rng.standard_normal((nV, 3))
        P = bg.fixed_point_constraint_matrix(V, fixed)
        R = oracle.fixed_point_constraint_matrix(nV, fixed)
        assert P.shape == R.shape
        assert np.array_equal(P.indptr, R.indptr) and np.array_equal(P.indices, R.indices)
        assert np.array_equal(P.data, R.data)


def test_fixed_point_constraint_rejects_unsorted():
    with pytest.raises(bg.BartelsError):
        bg.fixed_point_constraint_matrix(np.zeros((4, 3)), [2, 1])


def test_find_min_vertices_matches_oracle(oracle):
    V, E = kuhn_cube(3)
    for dim in range(3):
        assert np.array_equal(bg.find_min_vertices(V, dim), oracle.find_min_vertices(V, dim))


def _ref_linesearch(x, d, f, g, max_it, alpha, c, p):
    """src/linesearch_backtracking_bisection.cpp:17-30 restated."""
    it = 0
    while f(x + alpha * d) > f(x) + c * g @ d and it < max_it:
        alpha *= p
        it += 1
    return x + alpha * d, (1 if it == max_it else 0)


@pytest.mark.parametrize("max_it", [0, 3, 100])
def test_host_linesearch_matches_reference(max_it):
    rng = np.random.default_rng(1)
    A = rng.standard_normal((6, 6))
    A = A @ A.T + np.eye(6)
    b = rng.standard_normal(6)
    f = lambda x: 0.5 * x @ A @ x - b @ x
    x0 = rng.standard_normal(6)
    g = A @ x0 - b
    d = -8.0 * g  # overshooting direction forces backtracking
    x = x0.copy()
    st = bg.linesearch_backtracking_bisection(x, d, f, g, max_it, 1.0, 1e-4, 0.5)
    xr, sr = _ref_linesearch(x0.copy(), d, f, g, max_it, 1.0, 1e-4, 0.5)
    assert st == sr
    assert np.array_equal(x, xr)


@pytest.mark.parametrize("n", [1, 2, 3])
def test_kuhn_cube_counts_and_pattern(oracle, n):
    V, E = kuhn_cube(n)
    c = cube_counts(n)
    assert len(V) == c["nV"] and len(E) == c["nT"]
    vol = oracle.volume(V, E)
    assert np.allclose(vol, 1.0 / (6 * n ** 3), rtol=1e-12)
    M = oracle.mass_matrix(len(V), E, np.ones(len(E)), vol)
    assert M.nnz == c["nnz"]


def build_sim_shim_test():
    """g++ build of tests/sim_shim_test.cpp against include/bartels_sim.hpp and the library."""
    import subprocess
    out_dir = os.path.join(ROOT, "tests", "_build")
    os.makedirs(out_dir, exist_ok=True)
    exe = os.path.join(out_dir, "sim_shim_test")
    libdir = os.path.join(ROOT, "bartels_gb300", "lib")
    subprocess.check_call(["g++", "-std=c++17", "-O1", os.path.join(ROOT, "tests", "sim_shim_test.cpp"), "-I",
                           os.path.join(ROOT, "include"), "-L", libdir, "-lbartels_gpu", f"-Wl,-rpath,{libdir}",
                           "-o", exe])
    return exe


def test_sim_shim_compiles():
    assert os.path.exists(build_sim_shim_test())


def test_sim_plan_cache_keys_on_content_and_evicts():
    """The sim:: layer's plan cache with stand-in plans (no device needed)."""
    import subprocess
    out_dir = os.path.join(ROOT, "tests", "_build")
    os.makedirs(out_dir, exist_ok=True)
    exe = os.path.join(out_dir, "sim_plan_cache_test")
    subprocess.check_call(["g++", "-std=c++17", "-O1", "-Wall", os.path.join(ROOT, "tests", "sim_plan_cache_test.cpp"),
                           "-I", os.path.join(ROOT, "include"), "-o", exe])
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "plan cache ok" in r.stdout, r.stderr


def test_sim_host_parts_without_a_gpu():
    """sim:: routines that run on the host (tests/sim_host_test.cpp): compressed
    columns from row-ordered values, P in compressed columns, find_min_vertices,
    the host line search."""
    import subprocess
    out_dir = os.path.join(ROOT, "tests", "_build")
    os.makedirs(out_dir, exist_ok=True)
    exe = os.path.join(out_dir, "sim_host_test")
    libdir = os.path.join(ROOT, "bartels_gb300", "lib")
    subprocess.check_call(["g++", "-std=c++17", "-O1", os.path.join(ROOT, "tests", "sim_host_test.cpp"), "-I",
                           os.path.join(ROOT, "include"), "-L", libdir, "-lbartels_gpu", f"-Wl,-rpath,{libdir}",
                           "-o", exe])
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "sim host ok" in r.stdout, r.stderr
