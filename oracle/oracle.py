"""ctypes front end of the FP64 CPU oracle.

TEST INFRASTRUCTURE ONLY: the checker for the CUDA library. Only tests/,
``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg may import this
module; the product package never does.

Each wrapper names the reference routine it restates (see bartels_oracle.hpp
for the file:line citations). Array conventions follow the reference: V (nV,3),
E (nT,4) 0-based, q interleaved (3 nV), dphidX (nT,12), params (nT,2).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np
import scipy.sparse as sp

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")

NEOHOOKEAN, STVK, COROTATIONAL, NEOHOOKEAN_ISOCHORIC, ARAP, LINEAR_ELASTICITY = 0, 1, 2, 3, 4, 5
MODELS = {"neohookean": NEOHOOKEAN, "stvk": STVK, "corotational": COROTATIONAL,
          "neohookean_isochoric": NEOHOOKEAN_ISOCHORIC, "arap": ARAP, "linear_elasticity": LINEAR_ELASTICITY}


def build(force: bool = False) -> str:
    """Compile the oracle shared library with g++ (OpenMP for the baseline)."""
    srcs = [os.path.join(HERE, f) for f in ("oracle_capi.cpp", "oracle_baseline.cpp")]
    hdrs = [os.path.join(HERE, "bartels_oracle.hpp")]
    if not force and os.path.exists(LIB):
        newest = max(os.path.getmtime(p) for p in srcs + hdrs)
        if os.path.getmtime(LIB) >= newest:
            return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = ["g++", "-O3", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-fopenmp", "-o", tmp] + srcs
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        d, i, vp = C.POINTER(C.c_double), C.POINTER(C.c_int), C.c_void_p
        L.or_tetmesh_q.restype = C.c_double
        L.or_tetmesh_dq2.restype = vp
        L.or_mass_matrix.restype = vp
        L.or_fixed_point_constraint.restype = vp
        L.or_csr_nnz.restype = C.c_longlong
        L.or_psi.restype = C.c_double
        L.or_find_min_vertices.restype = C.c_int
        for name in ("or_csr_rows", "or_csr_nnz", "or_csr_free"):
            getattr(L, name).argtypes = [vp]
        L.or_csr_copy.argtypes = [vp, i, i, d]
        _lib = L
    return _lib


def _d(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(C.POINTER(C.c_double))


def _i(a):
    a = np.ascontiguousarray(a, dtype=np.int32)
    return a, a.ctypes.data_as(C.POINTER(C.c_int))


def _colmajor(a, dtype):
    return np.asfortranarray(a, dtype=dtype).ravel(order="F")


def _csr(h, ncols=None):
    L = lib()
    n = L.or_csr_rows(h)
    nnz = L.or_csr_nnz(h)
    rp = np.zeros(n + 1, np.int32)
    ci = np.zeros(nnz, np.int32)
    va = np.zeros(nnz, np.float64)
    L.or_csr_copy(h, rp.ctypes.data_as(C.POINTER(C.c_int)), ci.ctypes.data_as(C.POINTER(C.c_int)),
                  va.ctypes.data_as(C.POINTER(C.c_double)))
    L.or_csr_free(h)
    return sp.csr_matrix((va, ci, rp), shape=(n, ncols if ncols is not None else n))


def dphi_dX(V, E):
    """linear_tetmesh_dphi_dX -> (nT, 12)."""
    V = np.asarray(V, np.float64)
    E = np.asarray(E, np.int32)
    _, vp = _d(_colmajor(V, np.float64))
    Ec, ep = _i(_colmajor(E, np.int32))
    out = np.zeros(12 * len(E))
    _, op = _d(out)
    lib().or_dphi_dX(len(V), vp, len(E), ep, op)
    return out.reshape(12, len(E)).T.copy()


def volume(V, E):
    V = np.asarray(V, np.float64)
    E = np.asarray(E, np.int32)
    _, vp = _d(_colmajor(V, np.float64))
    _, ep = _i(_colmajor(E, np.int32))
    out = np.zeros(len(E))
    lib().or_volume(len(V), vp, len(E), ep, out.ctypes.data_as(C.POINTER(C.c_double)))
    return out


def _elem_args(E, q, dphidX, vol, params):
    Ec, ep = _i(_colmajor(E, np.int32))
    qa, qp = _d(q)
    da, dp = _d(_colmajor(dphidX, np.float64))
    va, vp = _d(vol)
    pa, pp = _d(_colmajor(params, np.float64))
    keep = (Ec, qa, da, va, pa)
    return keep, (ep, qp, dp, vp, pp)


def tetmesh_q(model, E, q, dphidX, vol, params):
    """linear_tetmesh_{model}_q -> scalar (serial element-order sum)."""
    keep, a = _elem_args(E, q, dphidX, vol, params)
    return lib().or_tetmesh_q(MODELS.get(model, model), len(E), *a)


def tetmesh_q_elements(model, E, q, dphidX, vol, params):
    keep, a = _elem_args(E, q, dphidX, vol, params)
    out = np.zeros(len(E))
    lib().or_tetmesh_q_elements(MODELS.get(model, model), len(E), *a, out.ctypes.data_as(C.POINTER(C.c_double)))
    return out


def tetmesh_dq(model, nV, E, q, dphidX, vol, params):
    """linear_tetmesh_{model}_dq -> (3 nV,)."""
    keep, a = _elem_args(E, q, dphidX, vol, params)
    g = np.zeros(3 * nV)
    lib().or_tetmesh_dq(MODELS.get(model, model), nV, len(E), *a, g.ctypes.data_as(C.POINTER(C.c_double)))
    return g


def tetmesh_dq2(model, nV, E, q, dphidX, vol, params, psd_tol=None, corot_layout_reference=True):
    """linear_tetmesh_{model}_dq2 (+ simple_psd_fix(tol) callback) -> scipy CSR."""
    keep, a = _elem_args(E, q, dphidX, vol, params)
    h = lib().or_tetmesh_dq2(MODELS.get(model, model), 0 if psd_tol is None else 1,
                             C.c_double(0.0 if psd_tol is None else psd_tol), int(corot_layout_reference),
                             nV, len(E), *a)
    return _csr(h)


def tetmesh_dq2_elements(model, E, q, dphidX, vol, params, psd_tol=None, corot_layout_reference=True):
    """Per-element 12x12 blocks (nT, 12, 12) (row = local dof a, col = local dof b)."""
    keep, a = _elem_args(E, q, dphidX, vol, params)
    out = np.zeros(144 * len(E))
    lib().or_tetmesh_dq2_elements(MODELS.get(model, model), 0 if psd_tol is None else 1,
                                  C.c_double(0.0 if psd_tol is None else psd_tol), int(corot_layout_reference),
                                  len(E), *a, out.ctypes.data_as(C.POINTER(C.c_double)))
    # stored column-major per element: out[t, a + 12 b] = K[a, b]
    return out.reshape(len(E), 12, 12).transpose(0, 2, 1).copy()


def mass_matrix(nV, E, density, vol):
    Ec, ep = _i(_colmajor(E, np.int32))
    da, dp = _d(density)
    va, vp = _d(vol)
    return _csr(lib().or_mass_matrix(nV, len(E), ep, dp, vp))


def const_ext_force(nV, E, vol, traction):
    Ec, ep = _i(_colmajor(E, np.int32))
    va, vp = _d(vol)
    ta, tp = _d(np.asarray(traction, np.float64))
    f = np.zeros(3 * nV)
    lib().or_const_ext_force(nV, len(E), ep, vp, tp, f.ctypes.data_as(C.POINTER(C.c_double)))
    return f


def fixed_point_constraint_matrix(nV, fixed, dim=3):
    fa, fp = _i(np.asarray(fixed, np.int32))
    return _csr(lib().or_fixed_point_constraint(nV, dim, fp, len(fa)), ncols=dim * nV)


def find_min_vertices(V, dim, tol=1e-3):
    V = np.asarray(V, np.float64)
    _, vp = _d(_colmajor(V, np.float64))
    out = np.zeros(len(V), np.int32)
    k = lib().or_find_min_vertices(len(V), vp, dim, C.c_double(tol), out.ctypes.data_as(C.POINTER(C.c_int)))
    return out[:k].copy()


def _f9(F):
    return _d(np.asarray(F, np.float64).ravel(order="F"))


def psi(model, F, p):
    Fa, fp = _f9(F)
    pa, pp = _d(p)
    return lib().or_psi(MODELS.get(model, model), fp, pp)


def dpsi(model, F, p):
    Fa, fp = _f9(F)
    pa, pp = _d(p)
    out = np.zeros(9)
    lib().or_dpsi(MODELS.get(model, model), fp, pp, out.ctypes.data_as(C.POINTER(C.c_double)))
    return out


def d2psi(model, F, p, corot_layout_reference=True):
    """9x9 in the reference's storage (column-major F flatten; see header)."""
    Fa, fp = _f9(F)
    pa, pp = _d(p)
    out = np.zeros(81)
    lib().or_d2psi(MODELS.get(model, model), fp, pp, int(corot_layout_reference),
                   out.ctypes.data_as(C.POINTER(C.c_double)))
    return out.reshape(9, 9, order="F")


def d2psi_corot_dsvd_literal(F, p):
    Fa, fp = _f9(F)
    pa, pp = _d(p)
    out = np.zeros(81)
    lib().or_d2psi_corot_dsvd_literal(fp, pp, out.ctypes.data_as(C.POINTER(C.c_double)))
    return out.reshape(9, 9, order="F")


def svd3(F):
    Fa, fp = _f9(F)
    U = np.zeros(9)
    S = np.zeros(3)
    Vm = np.zeros(9)
    P = C.POINTER(C.c_double)
    lib().or_svd3(fp, U.ctypes.data_as(P), S.ctypes.data_as(P), Vm.ctypes.data_as(P))
    return U.reshape(3, 3, order="F"), S, Vm.reshape(3, 3, order="F")


def psd_fix(A, tol=1e-6):
    A = np.asfortranarray(np.array(A, np.float64))
    n = A.shape[0]
    lib().or_psd_fix(A.ctypes.data_as(C.POINTER(C.c_double)), n, C.c_double(tol))
    return np.array(A)


def psd_fix_ql(A, tol=1e-6):
    """simple_psd_fix with the tridiagonal-QL eigen-solver of the timed CPU baseline."""
    A = np.asfortranarray(np.array(A, np.float64))
    ok = lib().or_psd_fix_ql(A.ctypes.data_as(C.POINTER(C.c_double)), A.shape[0], C.c_double(tol))
    if not ok:
        raise RuntimeError("QL iteration did not converge")
    return np.array(A)


def build_B(dphi12):
    da, dp = _d(np.asarray(dphi12, np.float64))
    out = np.zeros(108)
    lib().or_build_B(dp, out.ctypes.data_as(C.POINTER(C.c_double)))
    return out.reshape(9, 12, order="F")


def emu_to_lame(E, nu):
    """matlab/emu_to_lame.m:17-18."""
    lam = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu))
    mu = E / (2.0 * (1.0 + nu))
    return lam, mu
