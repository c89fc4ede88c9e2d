import ctypes as C
import os
import subprocess
import sys

import numpy as np
import pytest
import scipy.sparse as sp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(autouse=True)
def _torch_on_library_stream(request):
    """GPU tests run torch's ops on the default context's stream: the library
    enqueues on its own non-blocking stream, so inputs that torch writes
    (zeros, host copies, arithmetic) are then ordered with the library's
    kernels without a host synchronisation after every tensor op."""
    if request.node.get_closest_marker("gpu") is None:
        yield
        return
    try:
        import torch
        ok = torch.cuda.is_available()
    except ImportError:
        ok = False
    if not ok:
        yield
        return
    import bartels_gb300 as bg
    with torch.cuda.stream(bg.Context.default().torch_stream()):
        yield


def load_golden_mesh(name):
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    return g["V"].astype(np.float64), g["E"].astype(np.int32)


def load_golden_csr(name):
    m = np.load(os.path.join(GOLDEN, name + ".npz"))
    return sp.csr_matrix((m["val"], m["col"], m["row_ptr"]), shape=tuple(m["shape"]))


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as o
    o.build()
    return o


@pytest.fixture(scope="session")
def bunny():
    return load_golden_mesh("coarser_bunny")


_HARNESS = None


def devmath():
    """g++ build of tests/devmath_harness.cpp (the library's element math on the host)."""
    global _HARNESS
    if _HARNESS is None:
        out_dir = os.path.join(ROOT, "tests", "_build")
        os.makedirs(out_dir, exist_ok=True)
        so = os.path.join(out_dir, "libdevmath_harness.so")
        src = os.path.join(ROOT, "tests", "devmath_harness.cpp")
        hdr = os.path.join(ROOT, "bartels_gb300", "csrc", "devmath.cuh")
        if not os.path.exists(so) or os.path.getmtime(so) < max(os.path.getmtime(src), os.path.getmtime(hdr)):
            tmp = so + f".tmp{os.getpid()}"
            subprocess.check_call(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-x", "c++", src,
                                   "-I", os.path.join(ROOT, "bartels_gb300", "csrc"), "-o", tmp])
            os.replace(tmp, so)
        L = C.CDLL(so)
        L.dm_psi_d.restype = C.c_double
        L.dm_element_hessian_d.restype = C.c_int
        L.dm_element_hessian_f.restype = C.c_int
        _HARNESS = L
    return _HARNESS


def gpu_available():
    try:
        import bartels_gb300 as bg
        h = C.c_void_p()
        s = bg.lib().bartels_ctx_create(0, C.byref(h))
        if s == 0:
            bg.lib().bartels_ctx_destroy(h)
            return True
    except Exception:
        return False
    return False


def noisy_cube(n, amp=0.02, seed=0, stretch=None):
    from bartels_gb300.meshes import kuhn_cube
    V, E = kuhn_cube(n)
    rng = np.random.default_rng(seed)
    h = 1.0 / n
    q = V.copy()
    if stretch is not None:
        q = q * np.asarray(stretch)
    q = q + rng.uniform(-amp * h, amp * h, size=V.shape)
    return V, E, q.ravel()
