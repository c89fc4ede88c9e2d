"""Loader for the in-tree C-ABI library libbartels_gpu.so (include/bartels_gpu.h).

There is no CPU fallback: if the library is missing or no GPU is present,
calls raise ``BartelsError``.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libbartels_gpu.so")

OK = 0
E_INVALID_ARG, E_NONFINITE, E_NOT_CONVERGED, E_DEVICE, E_TIMEOUT, E_UNSUPPORTED, E_NO_DEVICE = 1, 2, 3, 4, 5, 6, 7
CONVERGED, MAX_ITERATIONS_REACHED = 0, 1
NEOHOOKEAN, STVK, COROTATIONAL, NEOHOOKEAN_ISOCHORIC, ARAP, LINEAR_ELASTICITY = 0, 1, 2, 3, 4, 5
PSD_NONE, PSD_SIMPLE_FIX = 0, 1
DQ2_COROT_EXACT = 1
PRECOND_BLOCK_JACOBI, PRECOND_LEARNED, PRECOND_MULTIGRID, PRECOND_LEARNED_MULTIGRID = 0, 1, 2, 3


class BartelsError(RuntimeError):
    def __init__(self, status, where, detail=""):
        self.status = status
        super().__init__(f"{where}: status {status} ({detail})")


class PcgParams(C.Structure):
    _fields_ = [("rel_tol", C.c_double), ("max_iters", C.c_int), ("inner_rel_tol", C.c_double),
                ("max_refinements", C.c_int), ("restart", C.c_int)]


class PcgReport(C.Structure):
    _fields_ = [("iterations", C.c_int), ("refinements", C.c_int), ("rel_residual", C.c_double),
                ("converged", C.c_int)]


class NewtonParams(C.Structure):
    _fields_ = [("model", C.c_int), ("psd_mode", C.c_int), ("psd_tol", C.c_double), ("dq2_flags", C.c_int),
                ("mass_coeff", C.c_double), ("scale", C.c_double), ("force_scale", C.c_double),
                ("gradient_tol", C.c_double), ("relative", C.c_int), ("max_iterations", C.c_int),
                ("max_iterations_ls", C.c_int), ("ls_alpha", C.c_double), ("ls_c", C.c_double),
                ("ls_p", C.c_double), ("pcg", PcgParams)]


class NewtonReport(C.Structure):
    _fields_ = [("status", C.c_int), ("iterations", C.c_int), ("pcg_iterations", C.c_int),
                ("ls_iterations", C.c_int), ("ls_failures", C.c_int), ("grad_norm0", C.c_double),
                ("grad_norm", C.c_double), ("energy", C.c_double), ("seconds", C.c_double),
                ("t_gradient", C.c_double), ("t_hessian", C.c_double), ("t_pcg", C.c_double),
                ("t_linesearch", C.c_double), ("last_alpha", C.c_double), ("last_pcg_rel_residual", C.c_double),
                ("last_pcg_iterations", C.c_int), ("last_pcg_refinements", C.c_int), ("pcg_failures", C.c_int),
                ("energy_change", C.c_double), ("precond_fallbacks", C.c_int), ("t_precond", C.c_double)]


OBJECTIVE_FN = C.CFUNCTYPE(C.c_double, C.POINTER(C.c_double), C.c_int, C.c_void_p)

_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int)
_P = C.c_void_p

# (name, restype, argtypes)
SIGNATURES = [
    ("bartels_status_string", C.c_char_p, [C.c_int]),
    ("bartels_last_error", C.c_char_p, []),
    ("bartels_ctx_create", C.c_int, [C.c_int, C.POINTER(_P)]),
    ("bartels_ctx_destroy", C.c_int, [_P]),
    ("bartels_ctx_synchronize", C.c_int, [_P]),
    ("bartels_ctx_stream", _P, [_P]),
    ("bartels_ctx_kernel_launches", C.c_int64, [_P]),
    ("bartels_tetmesh_dphi_dX", C.c_int, [_P, C.c_int, _D, C.c_int, _I, _D]),
    ("bartels_tetmesh_volume", C.c_int, [_P, C.c_int, _D, C.c_int, _I, _D]),
    ("bartels_plan_create", C.c_int, [_P, C.c_int, _D, C.c_int, _I, C.POINTER(_P)]),
    ("bartels_plan_destroy", C.c_int, [_P]),
    ("bartels_plan_set_element_data", C.c_int, [_P, _D, _D, _D, _D]),
    ("bartels_plan_csr_size", C.c_int, [_P, _I, C.POINTER(C.c_int64)]),
    ("bartels_plan_csr_pattern", C.c_int, [_P, _I, _I]),
    ("bartels_tetmesh_q", C.c_int, [_P, _P, C.c_int, _D, _D, _D, _D, _D]),
    ("bartels_tetmesh_dq", C.c_int, [_P, _P, C.c_int, _D, _D, _D, _D, _D]),
    ("bartels_tetmesh_dq2", C.c_int, [_P, _P, C.c_int, _D, _D, _D, _D, C.c_int, C.c_double, C.c_int, _D]),
    ("bartels_tetmesh_mass_matrix", C.c_int, [_P, _P, _D, _D, _D]),
    ("bartels_tetmesh_const_ext_force", C.c_int, [_P, _P, _D, _D, _D]),
    ("bartels_fixed_point_constraint_matrix", C.c_int, [C.c_int, C.c_int, _I, C.c_int, _I, _I, _I, _D]),
    ("bartels_find_min_vertices", C.c_int, [C.c_int, _D, C.c_int, C.c_double, _I, _I]),
    ("bartels_pcg_default_params", None, [C.POINTER(PcgParams)]),
    ("bartels_search_direction_newton_sparse", C.c_int,
     [_P, C.c_int, _I, _I, _D, _D, _D, C.POINTER(PcgParams), C.POINTER(PcgReport)]),
    ("bartels_linesearch_backtracking_bisection", C.c_int,
     [C.c_int, _D, _D, OBJECTIVE_FN, _P, _D, C.c_int, C.c_double, C.c_double, C.c_double, _I, _D]),
    ("bartels_newton_default_params", None, [C.POINTER(NewtonParams)]),
    ("bartels_newton_set_problem", C.c_int, [_P, _D, _D, _D, C.POINTER(C.c_ubyte)]),
    ("bartels_newton_solve", C.c_int, [_P, _P, C.POINTER(NewtonParams), _D, C.POINTER(NewtonReport)]),
    ("bartels_newton_solve_d", C.c_int, [_P, _P, C.POINTER(NewtonParams), _P, C.POINTER(NewtonReport)]),
    ("bartels_plan_hessian_d", C.c_int,
     [_P, _P, C.c_int, C.c_int, C.c_double, C.c_int, C.c_double, C.c_double, _P, _P]),
    ("bartels_plan_spmv_d", C.c_int, [_P, _P, _P, _P, _P]),
    ("bartels_newton_advance_implicit_euler_d", C.c_int, [_P, _P, C.c_double, _P]),
    ("bartels_tetmesh_dq_noalloc_d", C.c_int, [_P, _P, C.c_int, _P, _P]),
    ("bartels_lpcg_create", C.c_int, [_P, C.POINTER(_P)]),
    ("bartels_lpcg_destroy", C.c_int, [_P]),
    ("bartels_lpcg_num_params", C.c_int, []),
    ("bartels_lpcg_set_params", C.c_int, [_P, _P]),
    ("bartels_lpcg_get_params", C.c_int, [_P, _P, _P]),
    ("bartels_lpcg_train_step", C.c_int, [_P, _P, _P, _P, C.c_int, C.c_uint, C.c_float, C.c_float, _D]),
    ("bartels_lpcg_outputs", C.c_int, [_P, _P, _P, _P, _P]),
    ("bartels_plan_factor_size", C.c_int, [_P, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]),
    ("bartels_plan_set_preconditioner", C.c_int, [_P, C.c_int, _P]),
    ("bartels_plan_precond_apply_d", C.c_int, [_P, _P, _P, _P, _P, _I]),
    ("bartels_plan_mg_info", C.c_int, [_P, C.c_int, _I, _I, C.POINTER(C.c_int64), _I]),
    ("bartels_plan_pcg_d", C.c_int, [_P, _P, _P, _P, _P, C.POINTER(PcgParams), C.POINTER(PcgReport)]),
    ("bartels_newton_gradient_d", C.c_int, [_P, _P, C.POINTER(NewtonParams), _P, _P]),
    ("bartels_newton_energy_d", C.c_int, [_P, _P, C.POINTER(NewtonParams), _P, _D]),
    ("bartels_newton_get_problem", C.c_int, [_P, _D, _D]),
    ("bartels_plan_autotune", C.c_int, [_P, _P, _P, C.c_int, _I, _I]),
    ("bartels_segment_sumsq_d", C.c_int, [_P, C.c_int, _P, _P, _P]),
    ("bartels_plan_set_segments", C.c_int, [_P, C.c_int, _I, C.POINTER(C.c_int64)]),
    ("bartels_plan_autotune_hessian", C.c_int, [_P, _P, C.c_int, _P, C.c_int, _I, _I]),
    ("bartels_plan_pcg_spmv_time_d", C.c_int, [_P, _P, _P, _P, _P, C.c_int, C.POINTER(C.c_double)]),
    ("bartels_plan_set_hessian_tuning", C.c_int, [_P, C.c_int, C.c_int]),
    ("bartels_plan_set_segment_active", C.c_int, [_P, _P]),
    ("bartels_plan_segment_pcg_iterations", C.c_int, [_P, _I]),
    ("bartels_gemm_bf16_d", C.c_int, [_P, C.c_int, C.c_int, C.c_int, _P, C.c_int, _P, _P, C.c_int, _P, C.c_int]),
    ("bartels_gemm_bf16_wait_probe_d", C.c_int, [_P, C.c_int, C.c_int, C.c_int, _P, C.c_int, _P, _P, C.c_int, C.c_int]),
    ("bartels_newton_iterate_d", C.c_int,
     [_P, _P, C.POINTER(NewtonParams), _P, C.c_double, _I, C.POINTER(NewtonReport)]),
    ("bartels_tri_plan_create", C.c_int, [_P, C.c_int, C.c_int, _I, C.c_int, C.POINTER(_P)]),
    ("bartels_tri_plan_destroy", None, [_P]),
    ("bartels_tri_plan_csr_size", C.c_int, [_P, _I, C.POINTER(C.c_int64)]),
    ("bartels_tri_plan_csr_pattern", C.c_int, [_P, _I, _I]),
    ("bartels_tri2dmesh_dphi_dX", C.c_int, [_P, C.c_int, _D, C.c_int, _I, _D, _D]),
    ("bartels_tri2dmesh_q", C.c_int, [_P, _P, C.c_int, _D, _D, _D, _D, _D]),
    ("bartels_tri2dmesh_dq", C.c_int, [_P, _P, C.c_int, _D, _D, _D, _D, _D]),
    ("bartels_tri2dmesh_dq2", C.c_int, [_P, _P, C.c_int, _D, _D, _D, _D, C.c_int, C.c_double, _D]),
    ("bartels_tri2dmesh_mass_matrix", C.c_int, [_P, _P, _D, _D, _D]),
    ("bartels_tri3dmesh_dphi_dX", C.c_int, [_P, C.c_int, _D, C.c_int, _I, _D, _D]),
    ("bartels_tri3dmesh_stvk_dq2", C.c_int, [_P, _P, _D, _D, _D, _D, _D, _D, _D, C.c_int, C.c_double, _D]),
    ("bartels_pointwise_laws", C.c_int, [_P, C.c_int, C.c_int, _D, _D, _D, _D, _D]),
    ("bartels_tetmesh_q_d", C.c_int, [_P, _P, C.c_int, _P, _P]),
    ("bartels_plan_assemble_matrix", C.c_int, [_P, _P, _D, _D]),
    ("bartels_plan_assemble_vector", C.c_int, [_P, _P, _D, _D]),
    ("bartels_tetmesh_dq_d", C.c_int, [_P, _P, C.c_int, _P, _P]),
    ("bartels_tetmesh_q_elements_d", C.c_int, [_P, _P, C.c_int, _P, _P]),
    ("bartels_mex_routine_count", C.c_int, []),
    ("bartels_mex_routine_name", C.c_char_p, [C.c_int]),
    ("bartels_mex_release", None, []),
]


class MxArray(C.Structure):
    """bartels_mx of include/bartels_mex.h: an m x n column-major double matrix."""
    _fields_ = [("m", C.c_int64), ("n", C.c_int64), ("pr", _D)]


MX_ALLOC = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int64, C.c_int64, C.c_int64, C.POINTER(_D),
                       C.POINTER(C.POINTER(C.c_uint64)), C.POINTER(C.POINTER(C.c_uint64)))

_lib = None


def lib():
    """Load libbartels_gpu.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise BartelsError(E_UNSUPPORTED, "load",
                               f"{LIB_PATH} is missing; build it with `python -m bartels_gb300.build`")
        L = C.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(status, where):
    if status != OK:
        L = lib()
        detail = L.bartels_last_error().decode() or L.bartels_status_string(status).decode()
        raise BartelsError(status, where, detail)
    return status
