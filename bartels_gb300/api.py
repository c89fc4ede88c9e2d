"""Python mirror of the reference's mesh-level API over the C ABI.

Names, argument order and array conventions follow Bartels' ``sim::`` functions
(e.g. ``linear_tetmesh_neohookean_dq2(V, E, q, dphidX, volume, params)`` in
include/linear_tetmesh_neohookean_dq2.h:14-21). Sparse results are
``scipy.sparse.csr_matrix`` with the reference's assembled pattern (explicit
zeros kept). Every call runs on the GPU through libbartels_gpu.so; failures
raise ``BartelsError`` (the reference has no error returns: it asserts or
calls exit()).
"""
from __future__ import annotations

import atexit
import ctypes as C
import hashlib
import sys
import weakref
from collections import OrderedDict

import numpy as np
import scipy.sparse as sp

from . import _lib
from ._lib import BartelsError, check, lib

MODELS = {"neohookean": _lib.NEOHOOKEAN, "stvk": _lib.STVK, "corotational": _lib.COROTATIONAL,
          "neohookean_isochoric": _lib.NEOHOOKEAN_ISOCHORIC,
          "arap": _lib.ARAP, "linear_elasticity": _lib.LINEAR_ELASTICITY}


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _iptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _colmajor(a, dtype):
    return np.ascontiguousarray(np.asarray(a, dtype=dtype).ravel(order="F"))


class Context:
    """A device, a stream and workspace (bartels_ctx). Plans created on a
    context are destroyed before it (the C ABI requires that order)."""

    _default = None
    _live: "weakref.WeakSet[Context]" = weakref.WeakSet()

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        check(lib().bartels_ctx_create(device, C.byref(h)), "bartels_ctx_create")
        self.handle = h
        self.device = device
        self._plans: "weakref.WeakSet[MeshPlan]" = weakref.WeakSet()
        Context._live.add(self)

    @classmethod
    def default(cls) -> "Context":
        if cls._default is None:
            cls._default = Context(0)
        return cls._default

    def synchronize(self):
        check(lib().bartels_ctx_synchronize(self.handle), "bartels_ctx_synchronize")

    def torch_stream(self):
        """The context's CUDA stream as a torch stream. The library enqueues on
        its own non-blocking stream, so tensors that torch writes for a device
        call (or reads from one) are ordered with it by running those torch ops
        under `with torch.cuda.stream(ctx.torch_stream()):`."""
        if getattr(self, "_torch_stream", None) is None:
            import torch
            self._torch_stream = torch.cuda.ExternalStream(int(lib().bartels_ctx_stream(self.handle)),
                                                           device=f"cuda:{self.device}")
        return self._torch_stream

    @property
    def kernel_launches(self) -> int:
        return int(lib().bartels_ctx_kernel_launches(self.handle))

    def close(self):
        if self.handle:
            for p in list(self._plans):
                p.close()
            lib().bartels_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:
            pass


@atexit.register
def _close_all():
    """Destroy plans, then contexts, before the interpreter tears down."""
    for p in list(_plans.values()):
        p.close()
    _plans.clear()
    for c in list(Context._live):
        c.close()
    Context._default = None


class MeshPlan:
    """A mesh plan (bartels_mesh_plan): pattern, incidence lists, element data."""

    def __init__(self, V, E, ctx: Context | None = None):
        self.ctx = ctx or Context.default()
        self.V = _f64(V)
        self.E = np.ascontiguousarray(E, dtype=np.int32)
        if self.V.ndim != 2 or self.V.shape[1] != 3 or self.E.ndim != 2 or self.E.shape[1] != 4:
            raise BartelsError(_lib.E_INVALID_ARG, "MeshPlan", "V must be (nV,3) and E (nT,4)")
        self.nV, self.nT = len(self.V), len(self.E)
        vcm = _colmajor(self.V, np.float64)
        ecm = _colmajor(self.E, np.int32)
        h = C.c_void_p()
        check(lib().bartels_plan_create(self.ctx.handle, self.nV, _dptr(vcm), self.nT, _iptr(ecm), C.byref(h)),
              "bartels_plan_create")
        self.handle = h
        self.ctx._plans.add(self)
        n = C.c_int()
        nnz = C.c_int64()
        check(lib().bartels_plan_csr_size(h, C.byref(n), C.byref(nnz)), "bartels_plan_csr_size")
        self.n, self.nnz = n.value, nnz.value
        self._pattern = None

    def pattern(self):
        if self._pattern is None:
            rp = np.zeros(self.n + 1, np.int32)
            ci = np.zeros(self.nnz, np.int32)
            check(lib().bartels_plan_csr_pattern(self.handle, _iptr(rp), _iptr(ci)), "bartels_plan_csr_pattern")
            self._pattern = (rp, ci)
        return self._pattern

    def csr(self, values):
        rp, ci = self.pattern()
        return sp.csr_matrix((values, ci.copy(), rp.copy()), shape=(self.n, self.n))

    def set_element_data(self, dphidX=None, volume=None, params=None, density=None):
        keep = []

        def opt(a, cm=False):
            if a is None:
                return None
            arr = _colmajor(a, np.float64) if cm else _f64(np.ravel(a))
            keep.append(arr)
            return _dptr(arr)

        check(lib().bartels_plan_set_element_data(self.handle, opt(dphidX, True), opt(volume), opt(params, True),
                                                  opt(density)), "bartels_plan_set_element_data")

    # --- energy / gradient / Hessian ------------------------------------
    def _elem(self, dphidX, volume, params):
        keep = []
        out = []
        for a, cm in ((dphidX, True), (volume, False), (params, True)):
            if a is None:
                out.append(None)
            else:
                arr = _colmajor(a, np.float64) if cm else _f64(np.ravel(a))
                keep.append(arr)
                out.append(_dptr(arr))
        return keep, out

    def q(self, model, q, dphidX=None, volume=None, params=None) -> float:
        keep, (d, v, p) = self._elem(dphidX, volume, params)
        qa = _f64(q)
        e = C.c_double()
        check(lib().bartels_tetmesh_q(self.ctx.handle, self.handle, MODELS[model], _dptr(qa), d, v, p, C.byref(e)),
              "bartels_tetmesh_q")
        return e.value

    def dq(self, model, q, dphidX=None, volume=None, params=None):
        keep, (d, v, p) = self._elem(dphidX, volume, params)
        qa = _f64(q)
        g = np.zeros(3 * self.nV)
        check(lib().bartels_tetmesh_dq(self.ctx.handle, self.handle, MODELS[model], _dptr(qa), d, v, p, _dptr(g)),
              "bartels_tetmesh_dq")
        return g

    def dq2_values(self, model, q, dphidX=None, volume=None, params=None, psd_tol=None, corot_exact=False):
        keep, (d, v, p) = self._elem(dphidX, volume, params)
        qa = _f64(q)
        vals = np.zeros(self.nnz)
        psd = _lib.PSD_NONE if psd_tol is None else _lib.PSD_SIMPLE_FIX
        flags = _lib.DQ2_COROT_EXACT if corot_exact else 0
        check(lib().bartels_tetmesh_dq2(self.ctx.handle, self.handle, MODELS[model], _dptr(qa), d, v, p, psd,
                                        float(psd_tol or 0.0), flags, _dptr(vals)), "bartels_tetmesh_dq2")
        return vals

    def dq2(self, model, q, dphidX=None, volume=None, params=None, psd_tol=None, corot_exact=False):
        return self.csr(self.dq2_values(model, q, dphidX, volume, params, psd_tol, corot_exact))

    def mass_matrix(self, density, volume=None):
        d = _f64(np.ravel(density))
        v = None if volume is None else _f64(np.ravel(volume))
        vals = np.zeros(self.nnz)
        check(lib().bartels_tetmesh_mass_matrix(self.ctx.handle, self.handle, _dptr(d),
                                                None if v is None else _dptr(v), _dptr(vals)),
              "bartels_tetmesh_mass_matrix")
        return self.csr(vals)

    def assemble_matrix(self, Ke):
        """sim::assemble of caller-computed element matrices: Ke (nT, 12, 12),
        rows / columns 3a + k -> scipy CSR in the plan's pattern (FP64, summed in
        tet order as setFromTriplets sums the reference's triplets)."""
        K = np.ascontiguousarray(np.asarray(Ke, np.float64).reshape(self.nT, 12, 12).transpose(0, 2, 1))
        vals = np.zeros(self.nnz)
        check(lib().bartels_plan_assemble_matrix(self.ctx.handle, self.handle, _dptr(K), _dptr(vals)),
              "bartels_plan_assemble_matrix")
        return self.csr(vals)

    def assemble_vector(self, ge):
        """sim::assemble of caller-computed element vectors ge (nT, 12) -> (3 nV,)."""
        G = _f64(np.asarray(ge).reshape(self.nT, 12))
        g = np.zeros(3 * self.nV)
        check(lib().bartels_plan_assemble_vector(self.ctx.handle, self.handle, _dptr(G), _dptr(g)),
              "bartels_plan_assemble_vector")
        return g

    def const_ext_force(self, volume, traction):
        v = None if volume is None else _f64(np.ravel(volume))
        t = _f64(np.ravel(traction))
        f = np.zeros(3 * self.nV)
        check(lib().bartels_tetmesh_const_ext_force(self.ctx.handle, self.handle, None if v is None else _dptr(v),
                                                    _dptr(t), _dptr(f)), "bartels_tetmesh_const_ext_force")
        return f

    # --- Newton ---------------------------------------------------------------
    def set_problem(self, q_base=None, x_hat=None, f_ext=None, pinned=None):
        arrs = [None if a is None else _f64(a) for a in (q_base, x_hat, f_ext)]
        pin = None if pinned is None else np.ascontiguousarray(pinned, dtype=np.uint8)
        check(lib().bartels_newton_set_problem(
            self.handle, *[None if a is None else _dptr(a) for a in arrs],
            None if pin is None else pin.ctypes.data_as(C.POINTER(C.c_ubyte))), "bartels_newton_set_problem")

    def newton_solve(self, x, params: "_lib.NewtonParams"):
        xa = _f64(x).copy()
        rep = _lib.NewtonReport()
        check(lib().bartels_newton_solve(self.ctx.handle, self.handle, C.byref(params), _dptr(xa), C.byref(rep)),
              "bartels_newton_solve")
        return xa, rep

    def close(self):
        if getattr(self, "handle", None) and getattr(self.ctx, "handle", None):
            lib().bartels_plan_destroy(self.handle)
        self.handle = None

    def __del__(self):
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:
            pass


def newton_params(**kw) -> "_lib.NewtonParams":
    p = _lib.NewtonParams()
    lib().bartels_newton_default_params(C.byref(p))
    for k, v in kw.items():
        if k == "model" and isinstance(v, str):
            v = MODELS[v]
        if k in ("rel_tol", "max_iters", "inner_rel_tol", "max_refinements", "restart"):
            setattr(p.pcg, k, v)
        else:
            setattr(p, k, v)
    return p


# ---------------------------------------------------------------- drop-ins --
_plans: "OrderedDict[str, MeshPlan]" = OrderedDict()


def _plan_for(V, E) -> MeshPlan:
    V = _f64(V)
    E = np.ascontiguousarray(E, dtype=np.int32)
    key = hashlib.sha1(f"{V.shape}{E.shape}".encode() + V.tobytes() + E.tobytes()).hexdigest()
    p = _plans.get(key)
    if p is None:
        p = MeshPlan(V, E)
        _plans[key] = p
        while len(_plans) > 4:
            _plans.popitem(last=False)[1].close()
    else:
        _plans.move_to_end(key)
    return p


def linear_tetmesh_dphi_dX(V, E):
    """src/linear_tetmesh_dphi_dX.cpp:5-18 -> (nT, 12)."""
    V = np.asarray(V, np.float64)
    E = np.asarray(E, np.int32)
    vcm = _colmajor(V, np.float64)
    ecm = _colmajor(E, np.int32)
    out = np.zeros(12 * len(E))
    check(lib().bartels_tetmesh_dphi_dX(Context.default().handle, len(V), _dptr(vcm), len(E), _iptr(ecm),
                                        _dptr(out)), "bartels_tetmesh_dphi_dX")
    return out.reshape(12, len(E)).T.copy()


def volume(V, E):
    V = np.asarray(V, np.float64)
    E = np.asarray(E, np.int32)
    vcm = _colmajor(V, np.float64)
    ecm = _colmajor(E, np.int32)
    out = np.zeros(len(E))
    check(lib().bartels_tetmesh_volume(Context.default().handle, len(V), _dptr(vcm), len(E), _iptr(ecm),
                                       _dptr(out)), "bartels_tetmesh_volume")
    return out


def _make(model):
    def q_fn(V, E, q, dphidX, volume, params):
        return _plan_for(V, E).q(model, q, dphidX, volume, params)

    def dq_fn(V, E, q, dphidX, volume, params):
        return _plan_for(V, E).dq(model, q, dphidX, volume, params)

    def dq2_fn(V, E, q, dphidX, volume, params, psd_tol=None, corot_exact=False):
        return _plan_for(V, E).dq2(model, q, dphidX, volume, params, psd_tol, corot_exact)

    q_fn.__name__ = f"linear_tetmesh_{model}_q"
    dq_fn.__name__ = f"linear_tetmesh_{model}_dq"
    dq2_fn.__name__ = f"linear_tetmesh_{model}_dq2"
    return q_fn, dq_fn, dq2_fn


linear_tetmesh_neohookean_q, linear_tetmesh_neohookean_dq, linear_tetmesh_neohookean_dq2 = _make("neohookean")
linear_tetmesh_stvk_q, linear_tetmesh_stvk_dq, linear_tetmesh_stvk_dq2 = _make("stvk")
linear_tetmesh_corotational_q, linear_tetmesh_corotational_dq, linear_tetmesh_corotational_dq2 = _make(
    "corotational")
linear_tetmesh_arap_q, linear_tetmesh_arap_dq, linear_tetmesh_arap_dq2 = _make("arap")
linear_tetmesh_linear_elasticity_q, linear_tetmesh_linear_elasticity_dq, linear_tetmesh_linear_elasticity_dq2 = \
    _make("linear_elasticity")


# ------------------------------------------------------- 2D triangle meshes --
class Tri2DPlan:
    """A plan for a triangle mesh in the plane (bartels_tri_plan, 2 DOFs per
    vertex): the CSR pattern with 2x2 vertex blocks and the incidence lists."""

    DIM = 2

    def __init__(self, nV, E, ctx: Context | None = None):
        self.ctx = ctx or Context.default()
        self.E = np.ascontiguousarray(E, dtype=np.int32)
        if self.E.ndim != 2 or self.E.shape[1] != 3:
            raise BartelsError(_lib.E_INVALID_ARG, "Tri2DPlan", "E must be (nT,3)")
        self.nV, self.nT = int(nV), len(self.E)
        ecm = _colmajor(self.E, np.int32)
        h = C.c_void_p()
        check(lib().bartels_tri_plan_create(self.ctx.handle, self.nV, self.nT, _iptr(ecm), self.DIM, C.byref(h)),
              "bartels_tri_plan_create")
        self.handle = h
        self.ctx._plans.add(self)
        n = C.c_int()
        nnz = C.c_int64()
        check(lib().bartels_tri_plan_csr_size(h, C.byref(n), C.byref(nnz)), "bartels_tri_plan_csr_size")
        self.n, self.nnz = n.value, nnz.value
        rp = np.zeros(self.n + 1, np.int32)
        ci = np.zeros(self.nnz, np.int32)
        check(lib().bartels_tri_plan_csr_pattern(h, _iptr(rp), _iptr(ci)), "bartels_tri_plan_csr_pattern")
        self._pattern = (rp, ci)

    def pattern(self):
        return self._pattern

    def csr(self, values):
        rp, ci = self._pattern
        return sp.csr_matrix((values, ci.copy(), rp.copy()), shape=(self.n, self.n))

    def _args(self, q, dphidX, area, params):
        qa = _f64(np.ravel(q))
        if qa.size != 2 * self.nV:
            raise BartelsError(_lib.E_INVALID_ARG, "Tri2DPlan", "q must hold 2 nV values")
        keep = [qa, _colmajor(np.asarray(dphidX, np.float64).reshape(self.nT, 6), np.float64),
                _f64(np.ravel(area)), _colmajor(np.asarray(params, np.float64).reshape(self.nT, 2), np.float64)]
        return keep, [_dptr(a) for a in keep]

    def q(self, model, q, dphidX, area, params) -> float:
        keep, (qp, d, a, p) = self._args(q, dphidX, area, params)
        e = C.c_double()
        check(lib().bartels_tri2dmesh_q(self.ctx.handle, self.handle, MODELS[model], qp, d, a, p, C.byref(e)),
              "bartels_tri2dmesh_q")
        return e.value

    def dq(self, model, q, dphidX, area, params):
        keep, (qp, d, a, p) = self._args(q, dphidX, area, params)
        g = np.zeros(2 * self.nV)
        check(lib().bartels_tri2dmesh_dq(self.ctx.handle, self.handle, MODELS[model], qp, d, a, p, _dptr(g)),
              "bartels_tri2dmesh_dq")
        return g

    def dq2(self, model, q, dphidX, area, params, psd_tol=None):
        keep, (qp, d, a, p) = self._args(q, dphidX, area, params)
        vals = np.zeros(self.nnz)
        psd = _lib.PSD_NONE if psd_tol is None else _lib.PSD_SIMPLE_FIX
        check(lib().bartels_tri2dmesh_dq2(self.ctx.handle, self.handle, MODELS[model], qp, d, a, p, psd,
                                          0.0 if psd_tol is None else float(psd_tol), _dptr(vals)),
              "bartels_tri2dmesh_dq2")
        return self.csr(vals)

    def mass_matrix(self, density, area):
        dens = _f64(np.broadcast_to(np.asarray(density, np.float64), (self.nT,)))
        ar = _f64(np.ravel(area))
        vals = np.zeros(self.nnz)
        check(lib().bartels_tri2dmesh_mass_matrix(self.ctx.handle, self.handle, _dptr(dens), _dptr(ar), _dptr(vals)),
              "bartels_tri2dmesh_mass_matrix")
        return self.csr(vals)

    def close(self):
        if getattr(self, "handle", None) and getattr(self.ctx, "handle", None):
            lib().bartels_tri_plan_destroy(self.handle)
        self.handle = None

    def __del__(self):
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:
            pass


_tri_plans: "OrderedDict[str, Tri2DPlan]" = OrderedDict()


def _tri_plan_for(V, E) -> Tri2DPlan:
    E = np.ascontiguousarray(E, dtype=np.int32)
    nV = len(V)
    key = hashlib.sha1(f"{nV}{E.shape}".encode() + E.tobytes()).hexdigest()
    p = _tri_plans.get(key)
    if p is None:
        p = Tri2DPlan(nV, E)
        _tri_plans[key] = p
        while len(_tri_plans) > 4:
            _tri_plans.popitem(last=False)[1].close()
    else:
        _tri_plans.move_to_end(key)
    return p


def _tri_geometry(V, E):
    V = np.asarray(V, np.float64)
    E = np.asarray(E, np.int32)
    vcm = _colmajor(V, np.float64)
    ecm = _colmajor(E, np.int32)
    d = np.zeros(6 * len(E))
    a = np.zeros(len(E))
    check(lib().bartels_tri2dmesh_dphi_dX(Context.default().handle, len(V), _dptr(vcm), len(E), _iptr(ecm),
                                          _dptr(d), _dptr(a)), "bartels_tri2dmesh_dphi_dX")
    return d.reshape(6, len(E)).T.copy(), a


def linear_tri2dmesh_dphi_dX(V, E):
    """src/linear_tri2dmesh_dphi_dX.cpp:5-18 -> (nT, 6), the column-major flatten
    of each 3x2 gradient matrix."""
    return _tri_geometry(V, E)[0]


def triangle_areas(V, E):
    """Unsigned areas |det [x1 - x0, x2 - x0]| / 2 of a planar triangle mesh."""
    return _tri_geometry(V, E)[1]


def _make_tri(model):
    def q_fn(V, E, q, dphidX, area, params):
        return _tri_plan_for(V, E).q(model, q, dphidX, area, params)

    def dq_fn(V, E, q, dphidX, area, params):
        return _tri_plan_for(V, E).dq(model, q, dphidX, area, params)

    def dq2_fn(V, E, q, dphidX, area, params, psd_tol=None):
        return _tri_plan_for(V, E).dq2(model, q, dphidX, area, params, psd_tol)

    q_fn.__name__ = f"linear_tri2dmesh_{model}_q"
    dq_fn.__name__ = f"linear_tri2dmesh_{model}_dq"
    dq2_fn.__name__ = f"linear_tri2dmesh_{model}_dq2"
    return q_fn, dq_fn, dq2_fn


linear_tri2dmesh_neohookean_q, linear_tri2dmesh_neohookean_dq, linear_tri2dmesh_neohookean_dq2 = \
    _make_tri("neohookean")
linear_tri2dmesh_stvk_q, linear_tri2dmesh_stvk_dq, linear_tri2dmesh_stvk_dq2 = _make_tri("stvk")
linear_tri2dmesh_corotational_q, linear_tri2dmesh_corotational_dq, linear_tri2dmesh_corotational_dq2 = \
    _make_tri("corotational")
linear_tri2dmesh_arap_q, linear_tri2dmesh_arap_dq, linear_tri2dmesh_arap_dq2 = _make_tri("arap")
linear_tri2dmesh_linear_elasticity_dq2 = _make_tri("linear_elasticity")[2]


def linear_tri2dmesh_mass_matrix(V, E, density, area):
    """src/linear_tri2dmesh_mass_matrix.cpp."""
    return _tri_plan_for(V, E).mass_matrix(density, area)


# ---------------------------------------------------- triangles in space (3D) --
class Tri3DPlan(Tri2DPlan):
    """A plan for a triangle mesh in space (bartels_tri_plan, 3 DOFs per vertex)."""

    DIM = 3

    def stvk_dq2(self, q, dphidX, N, n, dndq, area, params, psd_tol=None):
        """linear_tri3dmesh_stvk_dq2: q (3 nV), dphidX (nT, 9), N and n (nT, 3),
        dndq (nT, 27), area (nT), params (nT, 2) = (lambda, mu)."""
        nT = self.nT
        keep = [_f64(np.ravel(q)), _colmajor(np.asarray(dphidX, np.float64).reshape(nT, 9), np.float64),
                _colmajor(np.asarray(N, np.float64).reshape(nT, 3), np.float64),
                _colmajor(np.asarray(n, np.float64).reshape(nT, 3), np.float64),
                _colmajor(np.asarray(dndq, np.float64).reshape(nT, 27), np.float64), _f64(np.ravel(area)),
                _colmajor(np.asarray(params, np.float64).reshape(nT, 2), np.float64)]
        if keep[0].size != 3 * self.nV:
            raise BartelsError(_lib.E_INVALID_ARG, "Tri3DPlan", "q must hold 3 nV values")
        vals = np.zeros(self.nnz)
        psd = _lib.PSD_NONE if psd_tol is None else _lib.PSD_SIMPLE_FIX
        check(lib().bartels_tri3dmesh_stvk_dq2(self.ctx.handle, self.handle, *[_dptr(a) for a in keep], psd,
                                               0.0 if psd_tol is None else float(psd_tol), _dptr(vals)),
              "bartels_tri3dmesh_stvk_dq2")
        return self.csr(vals)


_tri3_plans: "OrderedDict[str, Tri3DPlan]" = OrderedDict()


def _tri3_plan_for(V, E) -> Tri3DPlan:
    E = np.ascontiguousarray(E, dtype=np.int32)
    nV = len(V)
    key = hashlib.sha1(f"{nV}{E.shape}".encode() + E.tobytes()).hexdigest()
    p = _tri3_plans.get(key)
    if p is None:
        p = Tri3DPlan(nV, E)
        _tri3_plans[key] = p
        while len(_tri3_plans) > 4:
            _tri3_plans.popitem(last=False)[1].close()
    else:
        _tri3_plans.move_to_end(key)
    return p


def _tri3_geometry(V, E):
    V = np.asarray(V, np.float64)
    E = np.asarray(E, np.int32)
    vcm = _colmajor(V, np.float64)
    ecm = _colmajor(E, np.int32)
    d = np.zeros(9 * len(E))
    a = np.zeros(len(E))
    check(lib().bartels_tri3dmesh_dphi_dX(Context.default().handle, len(V), _dptr(vcm), len(E), _iptr(ecm),
                                          _dptr(d), _dptr(a)), "bartels_tri3dmesh_dphi_dX")
    return d.reshape(9, len(E)).T.copy(), a


def linear_tri3dmesh_dphi_dX(V, E):
    """src/linear_tri3dmesh_dphi_dX.cpp -> (nT, 9), the column-major flatten of each 3x3."""
    return _tri3_geometry(V, E)[0]


def triangle_areas_3d(V, E):
    """|e1 x e2| / 2 of the triangles of a mesh in space."""
    return _tri3_geometry(V, E)[1]


def triangle_normals(x, E):
    """Unit normals n = (x1 - x0) x (x2 - x0) / |.| of the triangles at positions x
    (nV x 3) and their derivatives with respect to the element DOFs [x0 x1 x2]:
    (n (nT, 3), dndq (nT, 27) as the column-major flatten of the 3x9 Jacobian),
    the per-element inputs of linear_tri3dmesh_stvk_dq2."""
    x = np.asarray(x, np.float64).reshape(-1, 3)
    E = np.asarray(E)
    e1, e2 = x[E[:, 1]] - x[E[:, 0]], x[E[:, 2]] - x[E[:, 0]]
    c = np.cross(e1, e2)
    r = np.linalg.norm(c, axis=1)
    n = c / r[:, None]

    def skew(v):
        z = np.zeros(len(v))
        return np.stack([np.stack([z, -v[:, 2], v[:, 1]], 1), np.stack([v[:, 2], z, -v[:, 0]], 1),
                         np.stack([-v[:, 1], v[:, 0], z], 1)], 1)
    P = (np.eye(3)[None] - n[:, :, None] * n[:, None, :]) / r[:, None, None]  # dn/dc
    dc1, dc2 = -skew(e2), skew(e1)  # dc/de1 = -[e2]x, dc/de2 = [e1]x
    J = np.zeros((len(E), 3, 9))
    J[:, :, 3:6] = P @ dc1
    J[:, :, 6:9] = P @ dc2
    J[:, :, 0:3] = -(J[:, :, 3:6] + J[:, :, 6:9])
    return n, J.transpose(0, 2, 1).reshape(len(E), 27)


def linear_tri3dmesh_stvk_dq2(V, E, q, dphidX, N, n, dndq, area, params, psd_tol=None):
    """src/linear_tri3dmesh_stvk_dq2.cpp: StVK membrane Hessian (scipy CSR)."""
    return _tri3_plan_for(V, E).stvk_dq2(q, dphidX, N, n, dndq, area, params, psd_tol)


def linear_tetmesh_mass_matrix(V, E, density, volume):
    """src/linear_tetmesh_mass_matrix.cpp:7-24."""
    return _plan_for(V, E).mass_matrix(density, volume)


def linear_tetmesh_const_ext_force(V, E, volume, traction):
    """src/linear_tetmesh_const_ext_force.cpp:5-18."""
    return _plan_for(V, E).const_ext_force(volume, traction)


def fixed_point_constraint_matrix(V, fixed_indices):
    """src/fixed_point_constraint_matrix.cpp:7-38 (fixed_indices sorted ascending)."""
    V = np.asarray(V)
    nV, dim = V.shape
    f = np.ascontiguousarray(fixed_indices, dtype=np.int32)
    rows = C.c_int()
    check(lib().bartels_fixed_point_constraint_matrix(nV, dim, _iptr(f), len(f), C.byref(rows), None, None, None),
          "bartels_fixed_point_constraint_matrix")
    rp = np.zeros(rows.value + 1, np.int32)
    ci = np.zeros(rows.value, np.int32)
    va = np.zeros(rows.value)
    check(lib().bartels_fixed_point_constraint_matrix(nV, dim, _iptr(f), len(f), C.byref(rows), _iptr(rp), _iptr(ci),
                                                      _dptr(va)), "bartels_fixed_point_constraint_matrix")
    return sp.csr_matrix((va, ci, rp), shape=(rows.value, nV * dim))


def find_min_vertices(V, dim, tol=1e-3):
    """src/find_min_vertices.cpp:5-21."""
    vcm = _colmajor(np.asarray(V, np.float64), np.float64)
    out = np.zeros(len(V), np.int32)
    cnt = C.c_int()
    check(lib().bartels_find_min_vertices(len(V), _dptr(vcm), dim, tol, _iptr(out), C.byref(cnt)),
          "bartels_find_min_vertices")
    return out[:cnt.value].copy()


def search_direction_newton_sparse(g, H, rel_tol=1e-8, max_iters=20000):
    """src/search_direction_newton_sparse.cpp:5-26: d = -H^{-1} g (PCG instead of SparseLU).
    Returns (d, ok, report); ok mirrors the reference's bool."""
    H = sp.csr_matrix(H)
    H.sort_indices()
    g = _f64(g)
    rp = np.ascontiguousarray(H.indptr, np.int32)
    ci = np.ascontiguousarray(H.indices, np.int32)
    va = _f64(H.data)
    d = np.zeros_like(g)
    prm = _lib.PcgParams()
    lib().bartels_pcg_default_params(C.byref(prm))
    prm.rel_tol = rel_tol
    prm.max_iters = max_iters
    rep = _lib.PcgReport()
    s = lib().bartels_search_direction_newton_sparse(Context.default().handle, len(g), _iptr(rp), _iptr(ci),
                                                     _dptr(va), _dptr(g), _dptr(d), C.byref(prm), C.byref(rep))
    if s not in (_lib.OK, _lib.E_NOT_CONVERGED):
        check(s, "bartels_search_direction_newton_sparse")
    return d, s == _lib.OK, rep


def linesearch_backtracking_bisection(x, d, f, g, max_iterations, alpha, c, p):
    """src/linesearch_backtracking_bisection.cpp:5-31 for a Python objective f(x).
    Updates x in place; returns CONVERGED or MAX_ITERATIONS_REACHED."""
    if x.dtype != np.float64 or not x.flags.c_contiguous:
        raise BartelsError(_lib.E_INVALID_ARG, "linesearch", "x must be a contiguous float64 array")
    dd = _f64(d)
    gg = _f64(g)

    @_lib.OBJECTIVE_FN
    def cb(ptr, n, user):
        return float(f(np.ctypeslib.as_array(ptr, shape=(n,)).copy()))

    status = C.c_int()
    a = C.c_double()
    check(lib().bartels_linesearch_backtracking_bisection(len(x), _dptr(x), _dptr(dd), cb, None, _dptr(gg),
                                                          max_iterations, alpha, c, p, C.byref(status), C.byref(a)),
          "bartels_linesearch_backtracking_bisection")
    return status.value


# ------------------------------------------------------------- pointwise laws --
def _flat_F(F):
    """(3, 3), (n, 3, 3) or (n, 9) rows of column-major flattens -> (n, 9), single?"""
    F = np.asarray(F, np.float64)
    if F.shape == (3, 3):
        return F.T.reshape(1, 9), True
    if F.ndim == 3 and F.shape[1:] == (3, 3):
        return F.transpose(0, 2, 1).reshape(len(F), 9), False
    if F.ndim == 2 and F.shape[1] == 9:
        return F, False
    raise BartelsError(_lib.E_INVALID_ARG, "pointwise_laws", "F must be (3,3), (n,3,3) or (n,9)")


def pointwise_laws(model, F, params, psi=True, dpsi=True, d2psi=True, ctx: Context | None = None):
    """psi(F), dpsi/dF and d2psi/dF2 of `model` at each F (bartels_pointwise_laws):
    psi (n,), dpsi (n, 9) in the column-major flatten of F, d2psi (n, 9, 9);
    params one (2,) row per F (ARAP: k, optionally alone). A single (3, 3) F
    gives unbatched results."""
    ctx = ctx or Context.default()
    Fm, single = _flat_F(F)
    n = len(Fm)
    P = np.asarray(params, np.float64).reshape(n, -1)
    if P.shape[1] == 1:
        P = np.c_[P, np.zeros(n)]
    Fc, Pc = _colmajor(Fm, np.float64), _colmajor(P[:, :2], np.float64)
    o_psi = np.zeros(n) if psi else None
    o_dpsi = np.zeros((9, n)) if dpsi else None      # n x 9 column-major
    o_d2 = np.zeros((n, 9, 9)) if d2psi else None    # block t column-major: [t, c, r]
    check(lib().bartels_pointwise_laws(ctx.handle, MODELS[model], n, _dptr(Fc), _dptr(Pc),
                                       None if o_psi is None else _dptr(o_psi),
                                       None if o_dpsi is None else _dptr(o_dpsi),
                                       None if o_d2 is None else _dptr(o_d2)), "bartels_pointwise_laws")
    out = (o_psi, None if o_dpsi is None else o_dpsi.T.copy(),
           None if o_d2 is None else o_d2.transpose(0, 2, 1).copy())
    if single:
        out = tuple(None if a is None else a[0] for a in out)
    return out


def _named_law(model):
    def psi_F(F, params):
        return pointwise_laws(model, F, params, dpsi=False, d2psi=False)[0]

    def dpsi_dF(F, params):
        return pointwise_laws(model, F, params, psi=False, d2psi=False)[1]

    def d2psi_dF2(F, params):
        return pointwise_laws(model, F, params, psi=False, dpsi=False)[2]
    return psi_F, dpsi_dF, d2psi_dF2


# src/psi_neohookean_F.cpp, src/dpsi_neohookean_dF.cpp, src/d2psi_neohookean_dF2.cpp and the StVK files
psi_neohookean_F, dpsi_neohookean_dF, d2psi_neohookean_dF2 = _named_law("neohookean")
psi_stvk_F, dpsi_stvk_dF, d2psi_stvk_dF2 = _named_law("stvk")
