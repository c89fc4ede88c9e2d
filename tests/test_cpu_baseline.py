"""The timed CPU baseline (oracle/oracle_baseline.cpp) against the checker:
its simple_psd_fix eigen-solver (Householder tridiagonalisation + implicit QL)
agrees with the checker's cyclic Jacobi, and its reference-structured
assembly (triplets, sort / compress) produces the checker's matrix."""
import numpy as np
import pytest

from conftest import noisy_cube

from bartels_gb300.meshes import material_params


def _sym(rng, n, eig):
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    return (Q * eig) @ Q.T


@pytest.mark.parametrize("n", [3, 6, 9, 12])
def test_ql_projection_matches_jacobi(oracle, n):
    rng = np.random.default_rng(n)
    cases = [rng.standard_normal((n, n)) for _ in range(20)]
    cases = [0.5 * (A + A.T) for A in cases]
    cases.append(_sym(rng, n, np.r_[np.full(n // 2, 2.0), np.full(n - n // 2, -1.0)]))  # repeated
    cases.append(_sym(rng, n, 1e6 * (1 + 1e-9 * rng.standard_normal(n))))              # clustered
    cases.append(_sym(rng, n, np.geomspace(1e-8, 1e8, n) * rng.choice([-1, 1], n)))   # graded, indefinite
    cases.append(np.diag(rng.standard_normal(n)))                                      # already diagonal
    cases.append(np.zeros((n, n)))
    for A in cases:
        for tol in (1e-6, 1e-3):
            P = oracle.psd_fix_ql(A, tol)
            R = oracle.psd_fix(A, tol)
            scale = max(np.abs(A).max(), tol)
            assert np.abs(P - R).max() <= 1e-12 * scale
            assert np.array_equal(P, P.T)
            assert np.linalg.eigvalsh(P).min() >= tol - 1e-12 * scale


def test_ql_projection_reads_the_lower_triangle(oracle):
    rng = np.random.default_rng(5)
    A = rng.standard_normal((12, 12))
    L = np.tril(A) + np.tril(A, -1).T
    assert np.abs(oracle.psd_fix_ql(A, 1e-6) - oracle.psd_fix(L, 1e-6)).max() <= 1e-12 * np.abs(L).max()


@pytest.mark.parametrize("model", ["neohookean", "stvk", "corotational"])
def test_faithful_assembly_matches_checker(oracle, model):
    V, E, q = noisy_cube(3, amp=0.2, seed=3, stretch=(1.1, 0.9, 1.0))
    params = material_params(model, len(E), 2e6, 0.45)
    dphi, vol = oracle.dphi_dX(V, E), oracle.volume(V, E)
    from oracle.baseline import faithful_dq2
    H = oracle.tetmesh_dq2(model, len(V), E, q, dphi, vol, params, psd_tol=1e-6)
    nnz, s, a = faithful_dq2(model, len(V), E, q, dphi, vol, params, 1e-6)
    assert nnz == H.nnz
    assert abs(a - abs(H.data).sum()) <= 1e-11 * abs(H.data).sum()
    assert abs(s - H.data.sum()) <= 1e-11 * abs(H.data).sum()
