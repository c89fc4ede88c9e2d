"""MATLAB-gateway facade on the GPU: every routine called with the arguments a
reference gateway receives (1-based E as doubles, column-major matrices)
against the FP64 oracle, with sparse results compared in MATLAB's
compressed-column layout (jc / ir bit-exact, values within the tolerance of
the C ABI entry point behind the routine: 1e-5 of the largest entry for the
FP32 tet Hessian, 1e-10 elsewhere). Also: the gateways' q - 1 shift changes
nothing beyond rounding, and the plan cache follows V and E."""
import numpy as np
import pytest
import scipy.sparse as sp

import bartels_gb300 as bg
from bartels_gb300 import mex
from bartels_gb300.meshes import material_params
from conftest import noisy_cube
from oracle import tri2d as T

pytestmark = pytest.mark.gpu

MODELS = ["neohookean", "stvk", "corotational", "arap"]


def same_csc(A, R):
    R = sp.csc_matrix(R)
    return A.shape == R.shape and np.array_equal(A.indptr, R.indptr) and np.array_equal(A.indices, R.indices)


def rel_max(A, R):
    return abs(sp.csc_matrix(A) - sp.csc_matrix(R)).max() / abs(R).max()


@pytest.fixture(scope="module")
def tet_case():
    V, E, q = noisy_cube(3, amp=0.2, seed=11, stretch=(1.1, 0.9, 1.0))
    return V, E, q


def test_tet_dphi_and_mass(oracle, tet_case):
    V, E, _ = tet_case
    d = mex.call("linear_tetmesh_dphi_dX", V, E + 1.0)
    d_ref = oracle.dphi_dX(V, E)
    assert d.shape == (len(E), 12) and np.abs(d - d_ref).max() <= 1e-12 * np.abs(d_ref).max()
    vol = oracle.volume(V, E)
    rho = np.random.default_rng(1).uniform(500, 1500, len(E))
    M = mex.call("linear_tetmesh_mass_matrix", V, E + 1.0, rho, vol)
    M_ref = oracle.mass_matrix(len(V), E, rho, vol)
    assert same_csc(M, M_ref) and rel_max(M, M_ref) <= 1e-12


@pytest.mark.parametrize("model", MODELS)
def test_tet_energy_gradient_hessian(oracle, tet_case, model):
    V, E, q = tet_case
    params = material_params(model, len(E), 2e6, 0.45)
    dphi, vol = oracle.dphi_dX(V, E), oracle.volume(V, E)
    args = (V, E + 1.0, q, dphi, vol, params)
    e = mex.call(f"linear_tetmesh_{model}_q", *args)
    e_ref = oracle.tetmesh_q(model, E, q, dphi, vol, params)
    assert e.shape == (1, 1) and abs(e[0, 0] - e_ref) <= 1e-10 * abs(e_ref)
    g = mex.call(f"linear_tetmesh_{model}_dq", *args)
    g_ref = oracle.tetmesh_dq(model, len(V), E, q, dphi, vol, params)
    assert g.shape == (3 * len(V), 1) and np.linalg.norm(g[:, 0] - g_ref) <= 1e-10 * np.linalg.norm(g_ref)
    # no 7th argument: no projection; any 7th argument: simple_psd_fix(1e-3)
    for extra, tol in (((), None), (("fixed",), 1e-3)):
        H = mex.call(f"linear_tetmesh_{model}_dq2", *args, *extra)
        H_ref = oracle.tetmesh_dq2(model, len(V), E, q, dphi, vol, params, psd_tol=tol)
        assert same_csc(H, H_ref), extra
        assert rel_max(H, H_ref) <= 1e-5, (extra, rel_max(H, H_ref))


def test_tet_linear_elasticity_ignores_a_seventh_argument(oracle, tet_case):
    V, E, q = tet_case
    params = material_params("linear_elasticity", len(E), 2e6, 0.45)
    dphi, vol = oracle.dphi_dX(V, E), oracle.volume(V, E)
    u = q - V.ravel()
    H_ref = oracle.tetmesh_dq2("linear_elasticity", len(V), E, u, dphi, vol, params)
    for extra in ((), ("x",)):
        H = mex.call("linear_tetmesh_linear_elasticity_dq2", V, E + 1.0, u, dphi, vol, params, *extra)
        assert same_csc(H, H_ref) and rel_max(H, H_ref) <= 1e-5


def test_arap_accepts_one_parameter_column(oracle, tet_case):
    V, E, q = tet_case
    k = material_params("arap", len(E), 2e6, 0.45)[:, :1]
    dphi, vol = oracle.dphi_dX(V, E), oracle.volume(V, E)
    e = mex.call("linear_tetmesh_arap_q", V, E + 1.0, q, dphi, vol, k)[0, 0]
    assert abs(e - oracle.tetmesh_q("arap", E, q, dphi, vol, np.c_[k, np.zeros_like(k)])) <= 1e-10 * abs(e)


def test_gateway_q_shift_is_a_translation(oracle, tet_case):
    """The reference's gateways read q through parse_rhs_index (q - 1): a rigid
    translation, which these energies ignore; the facade uses q as given."""
    V, E, q = tet_case
    params = material_params("neohookean", len(E), 2e6, 0.45)
    dphi, vol = oracle.dphi_dX(V, E), oracle.volume(V, E)
    args = (V, E + 1.0, q, dphi, vol, params)
    e_ref = oracle.tetmesh_q("neohookean", E, q - 1.0, dphi, vol, params)
    g_ref = oracle.tetmesh_dq("neohookean", len(V), E, q - 1.0, dphi, vol, params)
    H_ref = oracle.tetmesh_dq2("neohookean", len(V), E, q - 1.0, dphi, vol, params, psd_tol=1e-3)
    assert abs(mex.call("linear_tetmesh_neohookean_q", *args)[0, 0] - e_ref) <= 1e-10 * abs(e_ref)
    g = mex.call("linear_tetmesh_neohookean_dq", *args)[:, 0]
    assert np.linalg.norm(g - g_ref) <= 1e-9 * np.linalg.norm(g_ref)
    assert rel_max(mex.call("linear_tetmesh_neohookean_dq2", *args, 1.0), H_ref) <= 1e-5


def test_plan_cache_follows_the_mesh(oracle):
    """Five distinct meshes through the four-entry cache (the first is evicted),
    a hit on the second, then the first again (rebuilt); a scaled V with the
    same E gets its own plan. Every result against the oracle."""
    model = "stvk"
    cases = [noisy_cube(n, amp=0.1, seed=20 + n) for n in (2, 3, 2, 4, 5, 3)]
    cases[2] = (cases[2][0] * 1.3, cases[2][1], cases[2][2] * 1.3)  # same E as cases[0], scaled V
    results = []
    for V, E, q in cases + cases[:1]:
        params = material_params(model, len(E), 1e6, 0.4)
        dphi, vol = oracle.dphi_dX(V, E), oracle.volume(V, E)
        H = mex.call(f"linear_tetmesh_{model}_dq2", V, E + 1.0, q, dphi, vol, params)
        H_ref = oracle.tetmesh_dq2(model, len(V), E, q, dphi, vol, params)
        assert same_csc(H, H_ref) and rel_max(H, H_ref) <= 1e-5
        results.append(H)
    assert np.array_equal(results[0].data, results[-1].data)
    mex.release()
    V, E, q = cases[1]
    params = material_params(model, len(E), 1e6, 0.4)
    H = mex.call(f"linear_tetmesh_{model}_dq2", V, E + 1.0, q, oracle.dphi_dX(V, E), oracle.volume(V, E), params)
    assert np.array_equal(H.data, results[1].data)


# ------------------------------------------------------------------ triangles
def tri_cases():
    V, E = T.square_mesh(4, seed=3, jitter=0.25)
    A = np.array([[1.1, 0.1], [-0.15, 0.9]])
    yield V, E, (V @ A.T).ravel()


@pytest.mark.parametrize("model", MODELS)
def test_tri2d_routines(model):
    for V, E, q in tri_cases():
        d, ar = T.dphi_dX(V, E), T.area(V, E)
        p = material_params(model, len(E), 2e6, 0.45)
        args = (V, E + 1.0, q, d, ar, p)
        e = mex.call(f"linear_tri2dmesh_{model}_q", *args)[0, 0]
        e_ref = T.energy(model, E, q, d, ar, p)
        assert abs(e - e_ref) <= 1e-10 * abs(e_ref)
        g = mex.call(f"linear_tri2dmesh_{model}_dq", *args)
        g_ref = T.gradient(model, len(V), E, q, d, ar, p)
        assert g.shape == (2 * len(V), 1) and np.linalg.norm(g[:, 0] - g_ref) <= 1e-10 * np.linalg.norm(g_ref)
        for extra, tol in (((), None), ((1.0,), 1e-3)):
            H = mex.call(f"linear_tri2dmesh_{model}_dq2", *args, *extra)
            H_ref = T.hessian(model, len(V), E, q, d, ar, p, tol)
            assert same_csc(H, H_ref) and rel_max(H, H_ref) <= 1e-10


def test_tri2d_dphi_mass_and_linear_elasticity():
    V, E, q = next(tri_cases())
    d = mex.call("linear_tri2dmesh_dphi_dX", V, E + 1.0)
    assert d.shape == (len(E), 6) and np.abs(d - T.dphi_dX(V, E)).max() <= 1e-10 * np.abs(d).max()
    ar = T.area(V, E)
    rho = np.random.default_rng(4).uniform(1, 2, len(E))
    M = mex.call("linear_tri2dmesh_mass_matrix", V, E + 1.0, rho, ar)
    M_ref = T.mass_matrix(len(V), E, rho, ar)
    assert same_csc(M, M_ref) and rel_max(M, M_ref) <= 1e-12
    p = material_params("linear_elasticity", len(E), 2e6, 0.45)
    H = mex.call("linear_tri2dmesh_linear_elasticity_dq2", V, E + 1.0, q, d, ar, p)
    H_ref = T.hessian("linear_elasticity", len(V), E, q, d, ar, p)
    assert same_csc(H, H_ref) and rel_max(H, H_ref) <= 1e-10


def test_tri3d_routines():
    V2, E = T.square_mesh(4, seed=6, jitter=0.2)
    V = np.c_[V2, 0.2 * np.sin(2.0 * V2[:, 0]) * np.cos(1.5 * V2[:, 1])]
    x = V * np.array([1.1, 0.9, 1.0]) + 0.01 * np.random.default_rng(6).uniform(-1, 1, V.shape)
    d = mex.call("linear_tri3dmesh_dphi_dX", V, E + 1.0)
    d_ref = T.dphi_dX_3d(V, E)
    assert d.shape == (len(E), 9) and np.abs(d - d_ref).max() <= 1e-10 * np.abs(d_ref).max()
    ar = T.area_3d(V, E)
    p = material_params("stvk", len(E), 2e6, 0.45)
    N, _ = bg.triangle_normals(V, E)
    n, dndq = bg.triangle_normals(x, E)
    for extra, tol in (((), None), (("fixed",), 1e-3)):
        H = mex.call("linear_tri3dmesh_stvk_dq2", V, E + 1.0, x.ravel(), d_ref, N, n, dndq, ar, p, *extra)
        H_ref = T.stvk_hessian_3d(len(V), E, x.ravel(), d_ref, N, n, dndq, ar, p, tol)
        assert same_csc(H, H_ref) and rel_max(H, H_ref) <= 1e-10
