"""ctypes front end of the OpenMP FP64 CPU baseline (oracle_baseline.cpp).

Test infrastructure and CPU timing only: bench.py times it on the host cores as
the reference arm and the cpu_baseline field; the GPU library never uses it.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import oracle as o

D = C.POINTER(C.c_double)


def _lib():
    L = o.lib()
    if not hasattr(L, "_ob_ready"):
        L.ob_create.restype = C.c_void_p
        L.ob_create.argtypes = [C.c_int, D, C.c_int, C.POINTER(C.c_int)]
        L.ob_free.argtypes = [C.c_void_p]
        L.ob_nnz.restype = C.c_longlong
        L.ob_nnz.argtypes = [C.c_void_p]
        L.ob_set.argtypes = [C.c_void_p, C.c_int, D, D, D, D, D, C.POINTER(C.c_ubyte), C.c_double, C.c_double,
                             C.c_double, C.c_double]
        L.ob_energy.restype = C.c_double
        L.ob_energy.argtypes = [C.c_void_p, D]
        L.ob_gradient.argtypes = [C.c_void_p, D, D]
        L.ob_hessian.argtypes = [C.c_void_p, D, C.c_int, C.c_int, C.c_int]
        L.ob_pcg.restype = C.c_int
        L.ob_pcg.argtypes = [C.c_void_p, D, D, C.c_double, C.c_int, D]
        L.ob_newton_iteration.argtypes = [C.c_void_p, D, C.c_double, C.c_int, C.c_int, D]
        L.ob_threads.restype = C.c_int
        L.ob_set_threads.argtypes = [C.c_int]
        L.ob_faithful_dq2.restype = C.c_longlong
        L.ob_faithful_dq2.argtypes = [C.c_int, C.c_double, C.c_int, C.c_int, C.POINTER(C.c_int), D, D, D, D, D]
        L.ob_wtime.restype = C.c_double
        L._ob_ready = True
    return L


def _p(a):
    return a.ctypes.data_as(D)


def faithful_dq2(model, nV, E, q, dphidX, vol, params, psd_tol):
    """linear_tetmesh_{model}_dq2 in the reference's structure on one thread
    (per-tet dense blocks, simple_psd_fix, triplets, sort / compress).
    Returns (nnz, sum of values, sum of |values|)."""
    L = _lib()
    Ec = np.asfortranarray(E, np.int32).ravel(order="F")
    arrs = [np.ascontiguousarray(q, np.float64), np.asfortranarray(dphidX, np.float64).ravel(order="F"),
            np.ascontiguousarray(vol, np.float64), np.asfortranarray(params, np.float64).ravel(order="F")]
    sums = np.zeros(2)
    nnz = L.ob_faithful_dq2(o.MODELS[model], -1.0 if psd_tol is None else psd_tol, nV, len(E),
                            Ec.ctypes.data_as(C.POINTER(C.c_int)), *[_p(a) for a in arrs], _p(sums))
    return int(nnz), float(sums[0]), float(sums[1])


class CpuNewton:
    def __init__(self, V, E):
        L = _lib()
        self.L = L
        self.nV, self.nT = len(V), len(E)
        Vc = np.asfortranarray(V, np.float64).ravel(order="F")
        Ec = np.asfortranarray(E, np.int32).ravel(order="F")
        self.h = L.ob_create(self.nV, _p(Vc), self.nT, Ec.ctypes.data_as(C.POINTER(C.c_int)))

    def set(self, model, params, density, q_base, x_hat, f_ext, pinned, mass_coeff, scale, force_scale, psd_tol):
        self._keep = [np.asfortranarray(params, np.float64).ravel(order="F")] + [
            np.ascontiguousarray(a, np.float64) for a in (density, q_base, x_hat, f_ext)]
        pin = np.ascontiguousarray(pinned, np.uint8)
        self._keep.append(pin)
        self.L.ob_set(self.h, o.MODELS[model], *[_p(a) for a in self._keep[:5]],
                      pin.ctypes.data_as(C.POINTER(C.c_ubyte)), mass_coeff, scale, force_scale,
                      -1.0 if psd_tol is None else psd_tol)

    def energy(self, x):
        return self.L.ob_energy(self.h, _p(np.ascontiguousarray(x, np.float64)))

    def gradient(self, x):
        g = np.zeros(3 * self.nV)
        self.L.ob_gradient(self.h, _p(np.ascontiguousarray(x, np.float64)), _p(g))
        return g

    def hessian_range(self, x, t0, t1, clear=True):
        self.L.ob_hessian(self.h, _p(np.ascontiguousarray(x, np.float64)), t0, t1, int(clear))

    def pcg(self, b, x, rel_tol, max_it):
        rel = C.c_double()
        it = self.L.ob_pcg(self.h, _p(b), _p(x), rel_tol, max_it, C.byref(rel))
        return it, rel.value

    def newton_iteration(self, x, pcg_rel_tol=1e-8, pcg_max_it=20000, ls_max=100):
        st = np.zeros(8)
        self.L.ob_newton_iteration(self.h, _p(x), pcg_rel_tol, pcg_max_it, ls_max, _p(st))
        keys = ["grad_norm", "pcg_iterations", "ls_iterations", "t_gradient", "t_hessian", "t_pcg",
                "t_linesearch", "alpha"]
        return dict(zip(keys, st.tolist()))

    @property
    def threads(self):
        return self.L.ob_threads()

    def set_threads(self, n):
        self.L.ob_set_threads(int(n))

    def wtime(self):
        return self.L.ob_wtime()

    def close(self):
        if self.h:
            self.L.ob_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
