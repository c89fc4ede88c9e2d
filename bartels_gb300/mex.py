"""Python view of the MATLAB-gateway facade (include/bartels_mex.h).

``call(routine, *args)`` passes its arguments exactly as a MATLAB gateway of the
reference receives them (matlab/<routine>.cpp: double matrices, column-major,
E and fixed-vertex lists 1-based) and returns what the gateway would hand back:
a numpy array for dense results, a ``scipy.sparse.csc_matrix`` built from the
facade's jc / ir / pr arrays for sparse ones. Scripts written against the
reference's MATLAB functions translate line by line:

    H = linear_tetmesh_neohookean_dq2(V, T, q, dphidX, vol, params, 'fixed')   % MATLAB
    H = mex.call("linear_tetmesh_neohookean_dq2", V, T + 1, q, dphidX, vol, params, "fixed")
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import scipy.sparse as sp

from . import _lib

_D = C.POINTER(C.c_double)
_U = C.POINTER(C.c_uint64)


def _fn():
    L = _lib.lib()
    f = L.bartels_mex_call
    if f.argtypes is None:
        f.restype = C.c_int
        f.argtypes = [C.c_char_p, C.c_int, C.POINTER(_lib.MxArray), _lib.MX_ALLOC, C.c_void_p]
    return f


def routines():
    L = _lib.lib()
    return [L.bartels_mex_routine_name(i).decode() for i in range(L.bartels_mex_routine_count())]


def _as_mx(a):
    """Any argument as MATLAB would see it: a string becomes a char row (its
    contents are not read: only its presence counts), a vector a column."""
    if isinstance(a, str):
        a = np.array([float(ord(c)) for c in a]).reshape(1, -1)
    a = np.asarray(a, np.float64)
    if a.ndim == 0:
        a = a.reshape(1, 1)
    elif a.ndim == 1:
        a = a.reshape(-1, 1)
    elif a.ndim != 2:
        raise ValueError("arguments must be scalars, vectors or matrices")
    return np.asfortranarray(a)


def call(routine: str, *args):
    keep = [_as_mx(a) for a in args]
    mx = (_lib.MxArray * max(1, len(keep)))()
    for i, a in enumerate(keep):
        mx[i].m, mx[i].n = a.shape
        mx[i].pr = a.ctypes.data_as(_D)
    out = {}

    def alloc(_user, m, n, nnz, pr, ir, jc):
        if nnz < 0:
            buf = np.zeros((m, n), np.float64, order="F")
            out["dense"] = buf
            pr[0] = buf.ctypes.data_as(_D)
        else:
            out["pr"] = np.zeros(max(nnz, 1), np.float64)
            out["ir"] = np.zeros(max(nnz, 1), np.uint64)
            out["jc"] = np.zeros(n + 1, np.uint64)
            out["shape"] = (m, n)
            pr[0] = out["pr"].ctypes.data_as(_D)
            ir[0] = out["ir"].ctypes.data_as(_U)
            jc[0] = out["jc"].ctypes.data_as(_U)
        return 0

    cb = _lib.MX_ALLOC(alloc)
    _lib.check(_fn()(routine.encode(), len(keep), mx, cb, None), routine)
    if "dense" in out:
        return out["dense"]
    nnz = int(out["jc"][-1])
    return sp.csc_matrix((out["pr"][:nnz], out["ir"][:nnz].astype(np.int64), out["jc"].astype(np.int64)),
                         shape=out["shape"])


def release():
    """Drop the facade's cached plans and its context."""
    _lib.lib().bartels_mex_release()
