"""Triangle meshes on the GPU (linear_tri2dmesh_*, linear_tri3dmesh_*) against the FP64 CPU
restatement (oracle/tri2d.py): shape gradients and areas, energy, gradient,
Hessian (pattern bit-exact, values with and without simple_psd_fix), linear
elasticity, the mass matrix, the named drop-ins and the reference's 2D case."""
import numpy as np
import pytest
import scipy.sparse as sp

import bartels_gb300 as bg
from bartels_gb300.meshes import material_params
from oracle import tri2d as T

pytestmark = pytest.mark.gpu

MODELS = ["neohookean", "stvk", "corotational", "arap"]


def rel_max(A, B):
    A, B = sp.csr_matrix(A), sp.csr_matrix(B)
    return abs(A - B).max() / abs(B).max()


def same_pattern(A, B):
    return np.array_equal(A.indptr, B.indptr) and np.array_equal(A.indices, B.indices)


def cases():
    V, E = T.square_mesh(5, seed=1, jitter=0.25)
    rng = np.random.default_rng(2)
    yield "rest", V, E, V.ravel().copy()
    A = np.array([[1.15, 0.1], [-0.2, 0.85]])
    yield "sheared", V, E, (V @ A.T + 0.04 / 5 * rng.uniform(-1, 1, V.shape)).ravel()
    Rt = np.array([[0.0, -1.0], [1.0, 0.0]])  # rotated by 90 degrees and compressed
    yield "rotated", V, E, (0.8 * V @ Rt.T).ravel()


def test_dphi_and_area():
    V, E = T.square_mesh(6, seed=3, jitter=0.3)
    assert np.abs(bg.linear_tri2dmesh_dphi_dX(V, E) - T.dphi_dX(V, E)).max() <= 1e-10 * np.abs(T.dphi_dX(V, E)).max()
    assert np.allclose(bg.triangle_areas(V, E), T.area(V, E), rtol=1e-13, atol=0)


@pytest.mark.parametrize("model", MODELS)
def test_energy_and_gradient(model):
    for name, V, E, q in cases():
        d, ar = T.dphi_dX(V, E), T.area(V, E)
        p = material_params(model, len(E), 2e6, 0.45)
        plan = bg.Tri2DPlan(len(V), E)
        # relative, plus a floor for the rest state where both are rounding noise around 0
        e, e_ref = plan.q(model, q, d, ar, p), T.energy(model, E, q, d, ar, p)
        assert abs(e - e_ref) <= 1e-10 * abs(e_ref) + 1e-13 * p.max() * ar.sum(), (name, e, e_ref)
        g, g_ref = plan.dq(model, q, d, ar, p), T.gradient(model, len(V), E, q, d, ar, p)
        assert np.linalg.norm(g - g_ref) <= 1e-10 * np.linalg.norm(g_ref) + 1e-13 * p.max(), name
        plan.close()


@pytest.mark.parametrize("model", MODELS + ["linear_elasticity"])
@pytest.mark.parametrize("psd_tol", [None, 1e-6, 1e3])
def test_hessian(model, psd_tol):
    for name, V, E, q in cases():
        d, ar = T.dphi_dX(V, E), T.area(V, E)
        p = material_params(model, len(E), 2e6, 0.45)
        plan = bg.Tri2DPlan(len(V), E)
        H = plan.dq2(model, q, d, ar, p, psd_tol)
        H_ref = T.hessian(model, len(V), E, q, d, ar, p, psd_tol)
        assert same_pattern(H, H_ref), name
        assert rel_max(H, H_ref) <= 1e-10, (name, rel_max(H, H_ref))
        plan.close()


def test_mass_matrix_and_named_drop_ins():
    V, E, q = next(c for c in cases() if c[0] == "sheared")[1:]
    d, ar = T.dphi_dX(V, E), T.area(V, E)
    rho = np.linspace(900.0, 1100.0, len(E))
    M = bg.linear_tri2dmesh_mass_matrix(V, E, rho, ar)
    M_ref = T.mass_matrix(len(V), E, rho, ar)
    assert same_pattern(M, M_ref) and rel_max(M, M_ref) <= 1e-14
    p = material_params("stvk", len(E), 2e6, 0.45)
    plan = bg.Tri2DPlan(len(V), E)
    assert bg.linear_tri2dmesh_stvk_q(V, E, q, d, ar, p) == plan.q("stvk", q, d, ar, p)
    assert np.array_equal(bg.linear_tri2dmesh_stvk_dq(V, E, q, d, ar, p), plan.dq("stvk", q, d, ar, p))
    H1 = bg.linear_tri2dmesh_stvk_dq2(V, E, q, d, ar, p, psd_tol=1e-6)
    assert abs(H1 - plan.dq2("stvk", q, d, ar, p, 1e-6)).max() == 0.0
    ple = material_params("linear_elasticity", len(E), 2e6, 0.45)
    assert abs(bg.linear_tri2dmesh_linear_elasticity_dq2(V, E, q, d, ar, ple) -
               T.hessian("linear_elasticity", len(V), E, q, d, ar, ple)).max() <= 1e-9 * 2e6
    with pytest.raises(bg.BartelsError):
        plan.q("linear_elasticity", q, d, ar, ple)  # the reference has no tri2d linear-elasticity energy
    plan.close()


def test_reference_2d_case_has_zero_gradient_at_rest():
    """tests/test_constitutive_model.cpp:107-135: one triangle at rest."""
    V = np.array([[96.921, 44.047], [81.5, 37.5], [87.452, 31.207]])
    E = np.array([[0, 1, 2]], np.int32)
    params = np.array([[6.2069e+06, 6.8966e+05]])
    d = bg.linear_tri2dmesh_dphi_dX(V, E)
    g = bg.linear_tri2dmesh_corotational_dq(V, E, V.ravel(), d, np.array([68.002]), params)
    assert np.abs(g).max() <= 1e-6 * params.max()


# ---------------------------------------------------------- triangles in space
def curved_sheet(n=5, seed=6):
    V2, E = T.square_mesh(n, seed=seed, jitter=0.2)
    V = np.c_[V2, 0.2 * np.sin(2.0 * V2[:, 0]) * np.cos(1.5 * V2[:, 1])]
    rng = np.random.default_rng(seed)
    Rz = np.array([[0.96, -0.28, 0.0], [0.28, 0.96, 0.0], [0.0, 0.0, 1.0]])
    x = V @ Rz.T * np.array([1.1, 0.9, 1.0]) + 0.03 / n * rng.uniform(-1, 1, V.shape)
    return V, E, x


def test_tri3d_dphi_and_area():
    V, E, _ = curved_sheet()
    d = bg.linear_tri3dmesh_dphi_dX(V, E)
    d_ref = T.dphi_dX_3d(V, E)
    assert np.abs(d - d_ref).max() <= 1e-10 * np.abs(d_ref).max()
    assert np.allclose(bg.triangle_areas_3d(V, E), T.area_3d(V, E), rtol=1e-13, atol=0)


@pytest.mark.parametrize("psd_tol", [None, 1e-6, 1e3])
def test_tri3d_stvk_hessian(psd_tol):
    V, E, x = curved_sheet()
    d, ar = T.dphi_dX_3d(V, E), T.area_3d(V, E)
    p = material_params("stvk", len(E), 2e6, 0.45)
    N, _ = bg.triangle_normals(V, E)
    for name, pos in (("rest", V), ("deformed", x)):
        n, dndq = bg.triangle_normals(pos, E)
        H = bg.linear_tri3dmesh_stvk_dq2(V, E, pos.ravel(), d, N, n, dndq, ar, p, psd_tol=psd_tol)
        H_ref = T.stvk_hessian_3d(len(V), E, pos.ravel(), d, N, n, dndq, ar, p, psd_tol)
        assert same_pattern(H, H_ref), name
        assert rel_max(H, H_ref) <= 1e-10, (name, rel_max(H, H_ref))


def test_flat_membrane_matches_planar_stvk_on_the_gpu():
    V2, E = T.square_mesh(4, seed=4, jitter=0.2)
    V3 = np.c_[V2, np.zeros(len(V2))]
    x2 = V2 @ np.array([[1.1, 0.15], [-0.05, 0.95]]).T
    x3 = np.c_[x2, np.zeros(len(V2))]
    p = material_params("stvk", len(E), 1e5, 0.3)
    N, _ = bg.triangle_normals(V3, E)
    n, dndq = bg.triangle_normals(x3, E)
    H3 = bg.linear_tri3dmesh_stvk_dq2(V3, E, x3.ravel(), bg.linear_tri3dmesh_dphi_dX(V3, E), N, n, dndq,
                                      bg.triangle_areas_3d(V3, E), p).toarray()
    H2 = bg.linear_tri2dmesh_stvk_dq2(V2, E, x2.ravel(), bg.linear_tri2dmesh_dphi_dX(V2, E),
                                      bg.triangle_areas(V2, E), p).toarray()
    inplane = np.array([3 * v + k for v in range(len(V2)) for k in range(2)])
    assert np.abs(H3[np.ix_(inplane, inplane)] - H2).max() <= 1e-9 * np.abs(H2).max()
