"""GPU parity: every entry point through the C ABI against the FP64 oracle and
the reference's golden files.

Tolerances: FP64 paths (dphi_dX, volume, q, dq, mass, force) 1e-10 relative or
bit-exact where the operation order is the reference's; FP32 Hessians
1e-5 relative to the largest entry and to each row's own largest entry (per
element: tests/test_gpu_elements.py); CSR patterns bit-exact.
"""
import numpy as np
import pytest
import scipy.sparse as sp

import bartels_gb300 as bg
from bartels_gb300.meshes import kuhn_cube, material_params
from conftest import load_golden_csr, load_golden_mesh, noisy_cube

pytestmark = pytest.mark.gpu

MODELS = ["neohookean", "stvk", "corotational", "neohookean_isochoric", "arap", "linear_elasticity"]
HESS_TOL = 1e-5


def rel_max(A, B):
    A, B = sp.csr_matrix(A), sp.csr_matrix(B)
    return abs(A - B).max() / abs(B).max()


def rel_row(A, B, floor=1e-9):
    """Largest error of each row relative to that row's own largest entry (rows
    whose largest entry is below floor x the matrix's largest are measured
    against that floor), maximised over rows: small rows get no slack from
    large ones."""
    A, B = sp.csr_matrix(A), sp.csr_matrix(B)
    D = abs(A - B).tocsr()
    err = np.asarray(D.max(axis=1).todense()).ravel()
    scale = np.asarray(abs(B).max(axis=1).todense()).ravel()
    scale = np.maximum(scale, floor * scale.max())
    return float((err / scale).max())


def same_pattern(A, B):
    return np.array_equal(A.indptr, B.indptr) and np.array_equal(A.indices, B.indices)


def test_dphi_and_volume(oracle, bunny):
    V, E = bunny
    d = bg.linear_tetmesh_dphi_dX(V, E)
    d_ref = oracle.dphi_dX(V, E)
    assert np.abs(d - d_ref).max() <= 1e-12 * np.abs(d_ref).max()
    v = bg.volume(V, E)
    assert np.abs(v - oracle.volume(V, E)).max() <= 1e-12 * np.abs(v).max()


def test_golden_bunny_hessian_pattern_and_values(oracle, bunny):
    """data/matrices/H_neohookean_coarser_bunny.txt: pattern bit-exact, values
    (isochoric law, FP32 kernels) within 1e-5 of the reference's double path."""
    V, E = bunny
    H_ref = load_golden_csr("H_neohookean_coarser_bunny")
    YM, NU = 6e5, 0.4
    D = 0.5 * (YM * NU) / ((1.0 + NU) * (1.0 - 2.0 * NU))
    Cc = 0.5 * YM / (2.0 * (1.0 + NU))
    params = np.tile([Cc, D], (len(E), 1))
    q = (V * np.array([2.0, 4.0, 3.0])).ravel()
    dphi = oracle.dphi_dX(V, E)
    vol = oracle.volume(V, E)
    plan = bg.MeshPlan(V, E)
    H = plan.dq2("neohookean_isochoric", q, dphi, vol, params)
    assert same_pattern(H, H_ref)
    assert rel_max(H, H_ref) <= HESS_TOL
    assert rel_row(H, H_ref) <= HESS_TOL, rel_row(H, H_ref)
    assert sp.linalg.norm(H - H_ref) / sp.linalg.norm(H_ref) <= HESS_TOL
    # the drop-in name with the current law uses the same pattern
    H2 = bg.linear_tetmesh_neohookean_dq2(V, E, q, dphi, vol, params)
    assert same_pattern(H2, H_ref)


def test_golden_bunny_mass_and_force(oracle, bunny):
    V, E = bunny
    M_ref = load_golden_csr("M_coarse_bunny")
    vol = oracle.volume(V, E)
    M = bg.linear_tetmesh_mass_matrix(V, E, np.full(len(E), 0.1), vol)
    assert same_pattern(M, M_ref)
    assert sp.linalg.norm(M - M_ref) < 1e-8
    Mo = oracle.mass_matrix(len(V), E, np.full(len(E), 0.1), vol)
    assert np.array_equal(M.data, Mo.data)  # same operations, same order: bit-exact
    g = np.array([0, -9.8, 0])
    f = bg.linear_tetmesh_const_ext_force(V, E, vol, 0.1 * g)
    assert np.linalg.norm(f - M_ref @ np.tile(g, len(V))) < 1e-8
    assert np.array_equal(f, oracle.const_ext_force(len(V), E, vol, 0.1 * g))


def cases():
    yield "cube3", noisy_cube(3, amp=0.05, seed=1)
    V, E, q = noisy_cube(4, amp=0.3, seed=2, stretch=(1.1, 0.8, 1.05))
    yield "cube4_stretched", (V, E, q)


@pytest.mark.parametrize("model", MODELS)
def test_energy_gradient_fp64(oracle, model):
    for name, (V, E, q) in cases():
        params = material_params(model, len(E), 2e6, 0.45)
        dphi = oracle.dphi_dX(V, E)
        vol = oracle.volume(V, E)
        plan = bg.MeshPlan(V, E)
        e = plan.q(model, q, dphi, vol, params)
        e_ref = oracle.tetmesh_q(model, E, q, dphi, vol, params)
        assert abs(e - e_ref) <= 1e-10 * abs(e_ref), name
        g = plan.dq(model, q, dphi, vol, params)
        g_ref = oracle.tetmesh_dq(model, len(V), E, q, dphi, vol, params)
        assert np.linalg.norm(g - g_ref) <= 1e-10 * np.linalg.norm(g_ref), name


@pytest.mark.parametrize("model", MODELS)
@pytest.mark.parametrize("psd_tol", [None, 1e-6, 1e-3])
def test_hessian_fp32(oracle, model, psd_tol):
    for name, (V, E, q) in cases():
        params = material_params(model, len(E), 2e6, 0.45)
        dphi = oracle.dphi_dX(V, E)
        vol = oracle.volume(V, E)
        plan = bg.MeshPlan(V, E)
        H = plan.dq2(model, q, dphi, vol, params, psd_tol=psd_tol)
        H_ref = oracle.tetmesh_dq2(model, len(V), E, q, dphi, vol, params, psd_tol=psd_tol)
        assert same_pattern(H, H_ref), name
        assert rel_max(H, H_ref) <= HESS_TOL, (name, rel_max(H, H_ref))
        assert rel_row(H, H_ref) <= HESS_TOL, (name, rel_row(H, H_ref))


def test_arap_named_drop_ins_match_generic(oracle):
    V, E, q = noisy_cube(3, 0.01, 5)
    params = material_params("arap", len(E), 2e6, 0.45)
    dphi, vol = oracle.dphi_dX(V, E), oracle.volume(V, E)
    e = bg.linear_tetmesh_arap_q(V, E, q, dphi, vol, params)
    H = bg.linear_tetmesh_arap_dq2(V, E, q, dphi, vol, params, psd_tol=1e-6)
    assert abs(e - oracle.tetmesh_q("arap", E, q, dphi, vol, params)) <= 1e-10 * abs(e)
    H_ref = oracle.tetmesh_dq2("arap", len(V), E, q, dphi, vol, params, psd_tol=1e-6)
    assert same_pattern(H, H_ref) and rel_max(H, H_ref) <= HESS_TOL
    assert rel_row(H, H_ref) <= HESS_TOL, rel_row(H, H_ref)


def test_linear_elasticity_hessian_is_constant_and_gradient_linear(oracle):
    V, E, q = noisy_cube(3, 0.01, 6)
    params = material_params("linear_elasticity", len(E), 2e6, 0.45)
    dphi, vol = oracle.dphi_dX(V, E), oracle.volume(V, E)
    u = 1e-3 * np.random.default_rng(1).standard_normal(3 * len(V))
    H0 = bg.linear_tetmesh_linear_elasticity_dq2(V, E, u, dphi, vol, params)
    H1 = bg.linear_tetmesh_linear_elasticity_dq2(V, E, 2 * u + 1.0, dphi, vol, params)
    assert rel_max(H0, H1) <= 1e-6
    g = bg.linear_tetmesh_linear_elasticity_dq(V, E, u, dphi, vol, params)
    K = oracle.tetmesh_dq2("linear_elasticity", len(V), E, u, dphi, vol, params)
    assert np.linalg.norm(g - K @ u) <= 1e-10 * np.linalg.norm(g)


def test_corotational_exact_flag(oracle):
    V, E, q = noisy_cube(3, amp=0.3, seed=5, stretch=(1.2, 0.9, 1.0))
    params = material_params("corotational", len(E), 2e6, 0.45)
    dphi, vol = oracle.dphi_dX(V, E), oracle.volume(V, E)
    plan = bg.MeshPlan(V, E)
    H = plan.dq2("corotational", q, dphi, vol, params, corot_exact=True)
    H_ref = oracle.tetmesh_dq2("corotational", len(V), E, q, dphi, vol, params, corot_layout_reference=False)
    assert rel_max(H, H_ref) <= HESS_TOL
    assert rel_row(H, H_ref) <= HESS_TOL, rel_row(H, H_ref)


def test_psd_slow_path_on_compressed_mesh(oracle):
    """50% axial compression makes many StVK elements indefinite."""
    V, E, q = noisy_cube(3, amp=0.1, seed=6, stretch=(1.0, 1.0, 0.5))
    for model in ("stvk", "neohookean"):
        params = material_params(model, len(E), 1e6, 0.47)
        dphi, vol = oracle.dphi_dX(V, E), oracle.volume(V, E)
        plan = bg.MeshPlan(V, E)
        H = plan.dq2(model, q, dphi, vol, params, psd_tol=1e-6)
        H_ref = oracle.tetmesh_dq2(model, len(V), E, q, dphi, vol, params, psd_tol=1e-6)
        assert rel_max(H, H_ref) <= HESS_TOL
        assert rel_row(H, H_ref) <= HESS_TOL, rel_row(H, H_ref)
        assert np.linalg.eigvalsh(H.toarray()).min() > -1e-5 * abs(H).max()


def test_hessian_is_deterministic():
    V, E, q = noisy_cube(4, amp=0.1, seed=7)
    params = material_params("neohookean", len(E), 2e6, 0.45)
    plan = bg.MeshPlan(V, E)
    plan.set_element_data(params=params)
    a = plan.dq2_values("neohookean", q, psd_tol=1e-6)
    b = plan.dq2_values("neohookean", q, psd_tol=1e-6)
    assert np.array_equal(a, b)


def test_nonfinite_energy_is_an_error():
    V, E = kuhn_cube(1)
    q = V.copy()
    q[:, 2] *= -1.0  # inverted: J < 0, ln J undefined
    params = material_params("neohookean", len(E), 2e6, 0.45)
    with pytest.raises(bg.BartelsError):
        bg.linear_tetmesh_neohookean_q(V, E, q.ravel(), bg.linear_tetmesh_dphi_dX(V, E), bg.volume(V, E), params)


def test_search_direction_vs_direct_solve(oracle):
    V, E, q = noisy_cube(4, amp=0.05, seed=8)
    params = material_params("neohookean", len(E), 2e6, 0.45)
    dphi, vol = oracle.dphi_dX(V, E), oracle.volume(V, E)
    K = oracle.tetmesh_dq2("neohookean", len(V), E, q, dphi, vol, params, psd_tol=1e-6)
    M = oracle.mass_matrix(len(V), E, np.full(len(E), 1000.0), vol)
    fixed = oracle.find_min_vertices(V, 2)
    P = oracle.fixed_point_constraint_matrix(len(V), fixed)
    H = (P @ (M + 1e-4 * K) @ P.T).tocsr()
    g = np.random.default_rng(9).standard_normal(H.shape[0])
    d, ok, rep = bg.search_direction_newton_sparse(g, H)
    d_ref = -sp.linalg.spsolve(H.tocsc(), g)
    assert ok and rep.converged
    # the solve stops on the residual (1e-8 relative); the error is bounded by
    # cond(H) times that
    assert np.linalg.norm(H @ d + g) <= 1.01e-8 * np.linalg.norm(g)
    assert np.linalg.norm(d - d_ref) <= 1e-5 * np.linalg.norm(d_ref)


def _gravity_problem(n, model, nu=0.45):
    V, E, q = noisy_cube(n, amp=0.02, seed=0)
    rho = 1000.0
    params = material_params(model, len(E), 2e6, nu)
    fixed = bg.find_min_vertices(V, 2)
    pinned = np.zeros(len(V), np.uint8)
    pinned[fixed] = 1
    return V, E, q, params, rho, pinned


@pytest.mark.parametrize("n", [4, 8])
@pytest.mark.parametrize("model", ["neohookean", "stvk"])
def test_newton_quasistatic_vs_oracle(oracle, model, n):
    """Quasi-static solve of a gravity-loaded cube with z = 0 pinned, relative 1e-8
    (n = 8: the CPU-runnable configuration, 3,072 tets, E 2e6, nu 0.45, rho 1000,
    noise 0.02 h), against the oracle's Newton with a direct solve (SuperLU)."""
    from oracle import newton as on
    V, E, q, params, rho, pinned = _gravity_problem(n, model)
    vol = oracle.volume(V, E)
    fg = oracle.const_ext_force(len(V), E, vol, rho * np.array([0, 0, -9.81]))
    # unknown x = positions (pinned vertices keep q_base through the mask)
    q0 = q.copy()
    q_base = np.where(np.repeat(pinned, 3) == 1, q0, 0.0)
    x0 = np.where(np.repeat(pinned, 3) == 1, 0.0, q0)
    plan = bg.MeshPlan(V, E)
    plan.set_element_data(params=params, density=np.full(len(E), rho))
    plan.set_problem(q_base=q_base, f_ext=fg, pinned=pinned)
    prm = bg.newton_params(model=model, gradient_tol=1e-8, relative=1, mass_coeff=0.0, scale=1.0,
                           force_scale=1.0, max_iterations=50)
    x, rep = plan.newton_solve(x0, prm)
    assert rep.status == bg.CONVERGED
    obj = on.Objective(model, V, E, params, np.full(len(E), rho), q_base, None, fg, pinned, 0.0, 1.0, 1.0)
    xr = obj.P @ x0
    st, its = on.newtons_method_bisection(xr, obj.f, obj.grad, obj.hess, gradient_tol=1e-8, relative=True,
                                          max_iterations=50)
    assert st == on.CONVERGED
    xo = obj.P.T @ xr
    assert np.linalg.norm(x - xo) <= 1e-6 * np.linalg.norm(xo - np.where(np.repeat(pinned, 3) == 1, 0.0, V.ravel()))
    assert abs(rep.iterations - its) <= 2


def test_newton_implicit_euler_step_vs_oracle(oracle):
    """One implicit-Euler step (velocity form, PSD-projected Hessian)."""
    from oracle import newton as on
    model = "neohookean"
    V, E, q, params, rho, pinned = _gravity_problem(3, model)
    dt = 0.01
    vol = oracle.volume(V, E)
    fg = oracle.const_ext_force(len(V), E, vol, rho * np.array([0, 0, -9.81]))
    qt = V.ravel().copy()
    vt = np.zeros_like(qt)
    plan = bg.MeshPlan(V, E)
    plan.set_element_data(params=params, density=np.full(len(E), rho))
    plan.set_problem(q_base=qt, x_hat=vt, f_ext=fg, pinned=pinned)
    prm = bg.newton_params(model=model, psd_mode=bg.PSD_SIMPLE_FIX, psd_tol=1e-6, gradient_tol=1e-8, relative=1,
                           mass_coeff=1.0, scale=dt, force_scale=dt, max_iterations=30)
    v, rep = plan.newton_solve(np.zeros_like(qt), prm)
    assert rep.status == bg.CONVERGED
    obj = on.Objective(model, V, E, params, np.full(len(E), rho), qt, vt, fg, pinned, 1.0, dt, dt, psd_tol=1e-6)
    vr = np.zeros(obj.P.shape[0])
    st, its = on.newtons_method_bisection(vr, obj.f, obj.grad, obj.hess, gradient_tol=1e-8, relative=True,
                                          max_iterations=30)
    vo = obj.P.T @ vr
    assert np.linalg.norm(v - vo) <= 1e-6 * np.linalg.norm(vo)


def test_kernel_launch_counter():
    ctx = bg.Context.default()
    before = ctx.kernel_launches
    V, E = kuhn_cube(2)
    bg.linear_tetmesh_dphi_dX(V, E)
    assert ctx.kernel_launches > before


def test_device_hessian_and_spmv(oracle):
    """bartels_plan_hessian_d + bartels_plan_spmv_d (the PCG's SpMV row loop)."""
    torch = pytest.importorskip("torch")
    import ctypes as C
    from bartels_gb300 import _lib
    V, E, q = noisy_cube(4, amp=0.1, seed=10)
    params = material_params("neohookean", len(E), 2e6, 0.45)
    plan = bg.MeshPlan(V, E)
    plan.set_element_data(params=params, density=np.full(len(E), 1000.0))
    dphi, vol = oracle.dphi_dX(V, E), oracle.volume(V, E)
    K = oracle.tetmesh_dq2("neohookean", len(V), E, q, dphi, vol, params, psd_tol=1e-6)
    M = oracle.mass_matrix(len(V), E, np.full(len(E), 1000.0), vol)
    H = (M + 1e-4 * K).tocsr()
    L = bg.lib()
    qd = torch.from_numpy(q).cuda()
    x = torch.randn(3 * len(V), dtype=torch.float32, device="cuda")
    y = torch.empty_like(x)
    torch.cuda.synchronize()
    for lanes in (4, 8, 16):
        ctx = bg.Context(0)
        ctx_lanes = lanes
        import os
        os.environ["BARTELS_SPMV_LANES"] = str(ctx_lanes)
        ctx2 = bg.Context(0)
        plan2 = bg.MeshPlan(V, E, ctx2)
        plan2.set_element_data(params=params, density=np.full(len(E), 1000.0))
        _lib.check(L.bartels_plan_hessian_d(ctx2.handle, plan2.handle, _lib.NEOHOOKEAN, _lib.PSD_SIMPLE_FIX, 1e-6, 0,
                                            1e-4, 1.0, C.c_void_p(qd.data_ptr()), None), "hessian_d")
        _lib.check(L.bartels_plan_spmv_d(ctx2.handle, plan2.handle, None, C.c_void_p(x.data_ptr()),
                                         C.c_void_p(y.data_ptr())), "spmv_d")
        ctx2.synchronize()
        ref = H @ x.cpu().double().numpy()
        got = y.cpu().double().numpy()
        assert np.linalg.norm(got - ref) <= 1e-5 * np.linalg.norm(ref), lanes
        # the PCG loop's own SpMV over the padded copy of the values
        y.zero_()
        torch.cuda.synchronize()
        us = C.c_double()
        _lib.check(L.bartels_plan_pcg_spmv_time_d(ctx2.handle, plan2.handle, None, C.c_void_p(x.data_ptr()),
                                                  C.c_void_p(y.data_ptr()), 2, C.byref(us)), "pcg_spmv_time")
        ctx2.synchronize()
        got = y.cpu().double().numpy()
        assert np.linalg.norm(got - ref) <= 1e-5 * np.linalg.norm(ref), ("padded", lanes)
        assert us.value > 0
        plan2.close()
        ctx2.close()
        ctx.close()
    os.environ.pop("BARTELS_SPMV_LANES", None)


def test_sim_shim_cpp_program():
    """The C++ sim:: layer (include/bartels_sim.hpp) driven like the reference's headers."""
    import subprocess
    from test_capi import build_sim_shim_test
    r = subprocess.run([build_sim_shim_test()], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "sim shim ok" in r.stdout


def test_device_pointer_energy_and_gradient_match_host_forms():
    """bartels_tetmesh_q_d / _dq_d run the host forms' kernels on device data."""
    import ctypes as C
    import torch
    from bartels_gb300 import _lib
    from bartels_gb300.api import MODELS
    V, E, q = noisy_cube(4, amp=0.1, seed=12)
    L = bg.lib()
    for model in ("neohookean", "stvk", "corotational"):
        plan = bg.MeshPlan(V, E)
        plan.set_element_data(params=material_params(model, len(E), 2e6, 0.45))
        e, g = plan.q(model, q), plan.dq(model, q)
        qd = torch.from_numpy(q).cuda()
        ed = torch.zeros(1, dtype=torch.float64, device="cuda")
        gd = torch.zeros_like(qd)
        torch.cuda.synchronize()
        _lib.check(L.bartels_tetmesh_q_d(plan.ctx.handle, plan.handle, MODELS[model], C.c_void_p(qd.data_ptr()),
                                         C.c_void_p(ed.data_ptr())), "q_d")
        _lib.check(L.bartels_tetmesh_dq_d(plan.ctx.handle, plan.handle, MODELS[model], C.c_void_p(qd.data_ptr()),
                                          C.c_void_p(gd.data_ptr())), "dq_d")
        _lib.check(L.bartels_ctx_synchronize(plan.ctx.handle), "sync")
        assert ed.item() == e
        assert np.array_equal(gd.cpu().numpy(), g)
        plan.close()


def test_generic_assembly_matches_the_reference_bit_for_bit(oracle):
    """bartels_plan_assemble_matrix / _vector (the generic sim::assemble on
    caller-computed element quantities) reproduce the triplet assembly exactly."""
    V, E, q = noisy_cube(3, amp=0.1, seed=13, stretch=(1.0, 1.0, 0.8))
    params = material_params("stvk", len(E), 2e6, 0.45)
    dphi, vol = oracle.dphi_dX(V, E), oracle.volume(V, E)
    Ke = oracle.tetmesh_dq2_elements("stvk", E, q, dphi, vol, params, psd_tol=1e-6)
    H_ref = oracle.tetmesh_dq2("stvk", len(V), E, q, dphi, vol, params, psd_tol=1e-6)
    plan = bg.MeshPlan(V, E)
    H = plan.assemble_matrix(Ke)
    assert same_pattern(H, H_ref) and np.array_equal(H.data, H_ref.data)
    ge = np.random.default_rng(14).standard_normal((len(E), 12))
    g_ref = np.zeros(3 * len(V))
    for t in range(len(E)):            # the reference's order: element by element
        for a in range(4):
            g_ref[3 * E[t, a]:3 * E[t, a] + 3] += ge[t, 3 * a:3 * a + 3]
    assert np.array_equal(plan.assemble_vector(ge), g_ref)
    plan.close()


def test_search_direction_reports_an_iteration_cap(oracle):
    """A PCG solve stopped by max_iters returns the reference's `false`
    (BARTELS_E_NOT_CONVERGED underneath) with its residual, not a wrong d."""
    V, E, q = noisy_cube(4, amp=0.05, seed=8)
    params = material_params("neohookean", len(E), 2e6, 0.45)
    dphi, vol = oracle.dphi_dX(V, E), oracle.volume(V, E)
    K = oracle.tetmesh_dq2("neohookean", len(V), E, q, dphi, vol, params, psd_tol=1e-6)
    M = oracle.mass_matrix(len(V), E, np.full(len(E), 1000.0), vol)
    P = oracle.fixed_point_constraint_matrix(len(V), oracle.find_min_vertices(V, 2))
    H = (P @ (M + 1e-4 * K) @ P.T).tocsr()
    g = np.random.default_rng(9).standard_normal(H.shape[0])
    d, ok, rep = bg.search_direction_newton_sparse(g, H, max_iters=3)
    assert not ok and not rep.converged
    assert 0 < rep.iterations < 20 and rep.rel_residual > 1e-8
    d, ok, rep = bg.search_direction_newton_sparse(g, H)
    assert ok and rep.converged
