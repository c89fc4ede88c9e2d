"""The planar triangle-mesh restatement (oracle/tri2d.py) on the CPU: shape
function gradients, the reference's 2D known answer (zero corotational
gradient at rest, tests/test_constitutive_model.cpp:107-135), and finite
differences tying energy, gradient and Hessian together for every law."""
import numpy as np
import pytest

from bartels_gb300.meshes import material_params
from oracle import tri2d as T

MODELS = ["neohookean", "stvk", "corotational", "arap"]


def deformed(n=3, seed=0):
    V, E = T.square_mesh(n, seed=seed, jitter=0.2)
    rng = np.random.default_rng(seed + 1)
    A = np.array([[1.1, 0.2], [-0.1, 0.9]])
    q = (V @ A.T + 0.03 / n * rng.uniform(-1, 1, V.shape)).ravel()
    return V, E, q


def test_dphi_reproduces_linear_fields():
    V, E = T.square_mesh(4, seed=3, jitter=0.3)
    d = T.dphi_dX(V, E)
    rng = np.random.default_rng(0)
    a, c = rng.standard_normal(2), rng.standard_normal()
    f = V @ a + c
    for t, e in enumerate(E):
        phi = d[t].reshape(3, 2, order="F")
        assert np.allclose(phi.sum(axis=0), 0.0, atol=1e-12)
        assert np.allclose(f[e] @ phi, a, atol=1e-10)
    V0, E0 = T.square_mesh(4)
    assert np.isclose(T.area(V0, E0).sum(), 1.0, rtol=1e-12)


def test_reference_2d_case_has_zero_gradient_at_rest():
    """tests/test_constitutive_model.cpp:107-135: one triangle, q = rest positions."""
    V = np.array([[96.921, 44.047], [81.5, 37.5], [87.452, 31.207]])
    E = np.array([[0, 1, 2]])
    params = np.array([[6.2069e+06, 6.8966e+05]])
    g = T.gradient("corotational", 3, E, V.ravel(), T.dphi_dX(V, E), np.array([68.002]), params)
    assert np.abs(g).max() <= 1e-6 * params.max()


@pytest.mark.parametrize("model", MODELS)
def test_gradient_and_hessian_match_finite_differences(model):
    V, E, q = deformed()
    d, ar = T.dphi_dX(V, E), T.area(V, E)
    p = material_params(model, len(E), 1e5, 0.35)
    g = T.gradient(model, len(V), E, q, d, ar, p)
    # the exact Hessian (the reference stores the corotational one at F^T)
    H = T.hessian(model, len(V), E, q, d, ar, p, corot_layout_reference=False).toarray()
    rng = np.random.default_rng(7)
    h = 1e-6
    for _ in range(4):
        dq = rng.standard_normal(q.size)
        dq /= np.linalg.norm(dq)
        fd = (T.energy(model, E, q + h * dq, d, ar, p) - T.energy(model, E, q - h * dq, d, ar, p)) / (2 * h)
        assert abs(fd - g @ dq) <= 1e-6 * max(1.0, np.abs(g).sum()), (fd, g @ dq)
        fdg = (T.gradient(model, len(V), E, q + h * dq, d, ar, p) - T.gradient(model, len(V), E, q - h * dq, d, ar,
                                                                                p)) / (2 * h)
        assert np.linalg.norm(fdg - H @ dq) <= 1e-5 * np.linalg.norm(H @ dq), model


def test_linear_elasticity_hessian_is_the_second_derivative_of_the_strain_energy():
    """src/linear_tri2d_linear_elasticity_dq2.cpp: B^T C B area, with the plane-strain
    energy 1/2 e^T C e of the engineering strains checked by finite differences."""
    V, E, q = deformed(2)
    d, ar = T.dphi_dX(V, E), T.area(V, E)
    p = material_params("linear_elasticity", len(E), 1e5, 0.35)
    H = T.hessian("linear_elasticity", len(V), E, q, d, ar, p).toarray()
    assert np.allclose(H, H.T, atol=1e-9 * np.abs(H).max())
    # rigid translations are in the null space; a uniform stretch has energy 1/2 u^T H u = (lambda/2 + mu) s^2 |Omega| * 2
    u = np.tile([1.0, -2.0], len(V))
    assert np.abs(H @ u).max() <= 1e-9 * np.abs(H).max()
    lam, mu = 1e5 * 0.35 / (1.35 * 0.3), 1e5 / 2.7
    s = 1e-3
    u = (s * V).ravel()  # displacement s X: strain s I (plane strain)
    assert np.isclose(0.5 * u @ H @ u, (2 * mu + 2 * lam) * s * s * T.area(V, E).sum(), rtol=1e-9)


def test_mass_matrix_total_mass():
    V, E = T.square_mesh(3, seed=1, jitter=0.2)
    ar = T.area(V, E)
    rho = np.full(len(E), 7.0)
    M = T.mass_matrix(len(V), E, rho, ar)
    # each translation direction carries the total mass
    ux = np.tile([1.0, 0.0], len(V))
    assert np.isclose(ux @ M @ ux, 7.0 * ar.sum(), rtol=1e-12)


def test_flat_membrane_matches_the_planar_stvk_hessian():
    """A flat mesh in the xy plane under in-plane motion: the in-plane blocks of the
    3D membrane Hessian (src/linear_tri3d_stvk_dq2.cpp) are the planar StVK
    Hessian (F is the same embedded matrix with n = N = e_z)."""
    import bartels_gb300 as bg
    V2, E = T.square_mesh(2, seed=4, jitter=0.2)
    V3 = np.c_[V2, np.zeros(len(V2))]
    A = np.array([[1.1, 0.15], [-0.05, 0.95]])
    x2 = V2 @ A.T
    x3 = np.c_[x2, np.zeros(len(V2))]
    p = material_params("stvk", len(E), 1e5, 0.3)
    N, _ = bg.triangle_normals(V3, E)
    n, dndq = bg.triangle_normals(x3, E)
    H3 = T.stvk_hessian_3d(len(V3), E, x3.ravel(), T.dphi_dX_3d(V3, E), N, n, dndq, T.area_3d(V3, E), p).toarray()
    H2 = T.hessian("stvk", len(V2), E, x2.ravel(), T.dphi_dX(V2, E), T.area(V2, E), p).toarray()
    inplane = np.array([3 * v + k for v in range(len(V2)) for k in range(2)])
    assert np.abs(H3[np.ix_(inplane, inplane)] - H2).max() <= 1e-9 * np.abs(H2).max()
    assert np.allclose(T.area_3d(V3, E), T.area(V2, E), rtol=1e-13)
