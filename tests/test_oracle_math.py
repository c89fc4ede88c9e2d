"""Pin the oracle's constitutive math where no golden file exists: symbolic
differentiation of the reference's energy formulas, the reference's own
finite-difference scheme (src/finite_differences.cpp:42-80), numpy's SVD and
symmetric eigensolver, and the reference's literal dsvd route."""
import numpy as np
import pytest

PARAMS = {"neohookean": np.array([3.5e5, 1.2e6]), "neohookean_isochoric": np.array([3.5e5, 1.2e6]),
          "stvk": np.array([2.4e6, 7e5]), "corotational": np.array([2.4e6, 7e5])}


def rand_F(rng, amp=0.15):
    return np.eye(3) + amp * rng.standard_normal((3, 3))


def fd_grad(f, x, h=1e-6):
    g = np.zeros_like(x)
    for i in range(len(x)):
        xp = x.copy(); xp[i] += h
        xm = x.copy(); xm[i] -= h
        g[i] = (f(xp) - f(xm)) / (2 * h)
    return g


def fd_jac(fv, x, h=1e-6):
    J = np.zeros((len(fv(x)), len(x)))
    for i in range(len(x)):
        xp = x.copy(); xp[i] += h
        xm = x.copy(); xm[i] -= h
        J[:, i] = (fv(xp) - fv(xm)) / (2 * h)
    return J


@pytest.fixture(scope="module")
def sym():
    sy = pytest.importorskip("sympy")
    f = sy.symbols("f0:9")
    C, D = sy.symbols("C D")
    Fm = sy.Matrix(3, 3, lambda i, j: f[i + 3 * j])  # column-major flatten
    J = Fm.det()
    I1 = sum(x * x for x in f)
    E = (Fm.T * Fm - sy.eye(3)) / 2
    laws = {
        # src/psi_neohookean_F.cpp:31
        "neohookean": C * (I1 - 3 - 2 * sy.log(J)) + D * (J - 1) ** 2,
        # src/psi_neohookean_F.cpp:8-14 (commented-out isochoric law)
        "neohookean_isochoric": C * (J ** sy.Rational(-2, 3) * I1 - 3) + D * (J - 1) ** 2,
        # src/psi_stvk_F.cpp:11-12 with (lambda, mu) = (C, D)
        "stvk": D * (E * E).trace() + C / 2 * E.trace() ** 2,
    }
    out = {}
    for k, psi in laws.items():
        grad = [sy.diff(psi, x) for x in f]
        hess = [[sy.diff(g, x) for x in f] for g in grad]
        out[k] = (sy.lambdify([f, C, D], psi), sy.lambdify([f, C, D], grad), sy.lambdify([f, C, D], hess))
    return out


@pytest.mark.parametrize("model", ["neohookean", "neohookean_isochoric", "stvk"])
def test_laws_match_symbolic(oracle, sym, model):
    rng = np.random.default_rng(3)
    p = PARAMS[model]
    psi, grad, hess = sym[model]
    for _ in range(10):
        F = rand_F(rng)
        fv = F.ravel(order="F")
        e_ref = psi(fv, *p)
        assert abs(oracle.psi(model, F, p) - e_ref) <= 1e-12 * max(1.0, abs(e_ref))
        g_ref = np.array(grad(fv, *p), dtype=float)
        assert np.linalg.norm(oracle.dpsi(model, F, p) - g_ref) <= 1e-12 * np.linalg.norm(g_ref)
        H_ref = np.array(hess(fv, *p), dtype=float)
        assert np.linalg.norm(oracle.d2psi(model, F, p) - H_ref) <= 1e-12 * np.linalg.norm(H_ref)


@pytest.mark.parametrize("model", ["neohookean", "neohookean_isochoric", "stvk", "corotational"])
def test_gradient_and_hessian_by_finite_differences(oracle, model):
    rng = np.random.default_rng(4)
    p = PARAMS[model]
    for _ in range(5):
        F = rand_F(rng, 0.1)
        fv = F.ravel(order="F")
        e = lambda x: oracle.psi(model, x.reshape(3, 3, order="F"), p)
        g = lambda x: oracle.dpsi(model, x.reshape(3, 3, order="F"), p)
        gfd = fd_grad(e, fv)
        assert np.linalg.norm(g(fv) - gfd) <= 1e-6 * np.linalg.norm(gfd)
        Hfd = fd_jac(g, fv)
        H = oracle.d2psi(model, F, p, corot_layout_reference=False)
        assert np.linalg.norm(H - Hfd) <= 1e-5 * np.linalg.norm(Hfd)


def test_corotational_reference_layout_is_hessian_at_transpose(oracle):
    rng = np.random.default_rng(5)
    p = PARAMS["corotational"]
    for _ in range(10):
        F = rand_F(rng, 0.3)
        Href = oracle.d2psi("corotational", F, p, corot_layout_reference=True)
        Ht = oracle.d2psi("corotational", F.T, p, corot_layout_reference=False)
        assert np.linalg.norm(Href - Ht) <= 1e-10 * np.linalg.norm(Ht)
        # and it is not the Hessian at F for a generic F
        H = oracle.d2psi("corotational", F, p, corot_layout_reference=False)
        assert np.linalg.norm(Href - H) > 1e-3 * np.linalg.norm(H)


def test_corotational_reference_layout_matches_literal_dsvd(oracle):
    """Eigen-system form == the reference's dU/dS/dV route when the singular
    values are distinct (no perturbation needed there)."""
    rng = np.random.default_rng(6)
    p = PARAMS["corotational"]
    n = 0
    while n < 10:
        F = rand_F(rng, 0.4)
        U, S, Vt = np.linalg.svd(F)
        if np.min(np.abs(np.diff(np.sort(S)))) < 0.05 or np.linalg.det(F) <= 0:
            continue
        n += 1
        A = oracle.d2psi("corotational", F, p, corot_layout_reference=True)
        B = oracle.d2psi_corot_dsvd_literal(F, p)
        assert np.linalg.norm(A - B) <= 1e-9 * np.linalg.norm(B)


def test_corotational_repeated_singular_values_limit(oracle):
    """At F = I (all singular values equal) the reference perturbs F by 1e-5;
    the exact limit is the linear-elasticity tensor: 2 mu sym + lambda tr."""
    lam, mu = PARAMS["corotational"]
    H = oracle.d2psi("corotational", np.eye(3), PARAMS["corotational"])
    ref = np.zeros((9, 9))
    for i in range(3):
        for j in range(3):
            for k in range(3):
                for l in range(3):
                    ref[i + 3 * j, k + 3 * l] = (mu * ((i == k) * (j == l) + (i == l) * (j == k))
                                                 + lam * (i == j) * (k == l))
    assert np.linalg.norm(H - ref) <= 1e-9 * np.linalg.norm(ref)


def test_svd3_against_numpy(oracle):
    rng = np.random.default_rng(7)
    for k in range(50):
        F = rng.standard_normal((3, 3)) if k % 2 else rand_F(rng, 0.5)
        U, S, V = oracle.svd3(F)
        assert np.linalg.norm(U @ np.diag(S) @ V.T - F) <= 1e-12 * np.linalg.norm(F)
        assert np.linalg.det(U) > 0 and np.linalg.det(V) > 0
        assert np.allclose(U.T @ U, np.eye(3), atol=1e-12) and np.allclose(V.T @ V, np.eye(3), atol=1e-12)
        assert S[0] >= S[1] >= abs(S[2]) - 1e-14 and S[1] >= 0
        assert np.sign(S[2]) == np.sign(np.linalg.det(F))
        assert np.allclose(np.sort(np.abs(S)), np.sort(np.linalg.svd(F, compute_uv=False)), rtol=1e-12)


def test_psd_fix_against_numpy(oracle):
    rng = np.random.default_rng(8)
    for tol in (1e-6, 1e-3, 0.5):
        A = rng.standard_normal((12, 12))
        A = A + A.T
        w, Q = np.linalg.eigh(A)
        ref = Q @ np.diag(np.maximum(w, tol)) @ Q.T
        assert np.linalg.norm(oracle.psd_fix(A, tol) - ref) <= 1e-11 * np.linalg.norm(ref)


def test_fixed_point_constraint_matrix(oracle):
    nV = 7
    fixed = [0, 3, 6]
    P = oracle.fixed_point_constraint_matrix(nV, fixed).toarray()
    keep = [v for v in range(nV) if v not in fixed]
    ref = np.zeros((3 * len(keep), 3 * nV))
    for r, v in enumerate(keep):
        ref[3 * r:3 * r + 3, 3 * v:3 * v + 3] = np.eye(3)
    assert np.array_equal(P, ref)


def test_find_min_vertices(oracle):
    V = np.array([[0, 0, 0.0], [1, 0, 0.0005], [0, 1, 0.2], [1, 1, -0.0004]])
    assert list(oracle.find_min_vertices(V, 2)) == [0, 1, 3]
