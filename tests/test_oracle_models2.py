"""ARAP and linear elasticity in the FP64 restatement: ARAP against its own
stretch definition and finite differences; linear elasticity against the
closed form mu e:e + lambda/2 tr(e)^2 (e = sym(F)) and finite differences."""
import numpy as np
import pytest

from oracle import oracle as o


def fd_grad(f, x, h=1e-6):
    g = np.zeros_like(x)
    for i in range(len(x)):
        e = np.zeros_like(x)
        e[i] = h
        g[i] = (f(x + e) - f(x - e)) / (2 * h)
    return g


def test_arap_psi_is_sum_of_squared_stretch_deviations():
    rng = np.random.default_rng(0)
    for _ in range(20):
        F = np.eye(3) + 0.3 * rng.standard_normal((3, 3))
        if np.linalg.det(F) <= 0:
            continue
        s = np.linalg.svd(F, compute_uv=False)
        k = 2.5
        assert abs(o.psi("arap", F, np.array([k, 7.0])) - k * np.sum((s - 1) ** 2)) <= 1e-10 * max(1, k)


def test_linear_elasticity_closed_form():
    rng = np.random.default_rng(1)
    YM, nu = 3e5, 0.3
    lam, mu = YM * nu / ((1 + nu) * (1 - 2 * nu)), YM / (2 * (1 + nu))
    for _ in range(10):
        F = 0.2 * rng.standard_normal((3, 3))
        e = 0.5 * (F + F.T)
        ref = mu * np.sum(e * e) + 0.5 * lam * np.trace(e) ** 2
        assert abs(o.psi("linear_elasticity", F, np.array([YM, nu])) - ref) <= 1e-9 * abs(ref)
        P = o.dpsi("linear_elasticity", F, np.array([YM, nu]))
        Pref = 2 * mu * e + lam * np.trace(e) * np.eye(3)
        assert np.allclose(P, Pref.ravel(order="F"), rtol=1e-12, atol=1e-9)


@pytest.mark.parametrize("model,p", [("arap", np.array([1.7, 0.0])), ("linear_elasticity", np.array([2e3, 0.35]))])
def test_gradient_and_hessian_finite_differences(model, p):
    rng = np.random.default_rng(2)
    for _ in range(5):
        F0 = np.eye(3) + 0.2 * rng.standard_normal((3, 3))
        f = lambda v: o.psi(model, v.reshape(3, 3, order="F"), p)
        x0 = F0.ravel(order="F")
        g = o.dpsi(model, F0, p)
        assert np.allclose(g, fd_grad(f, x0), rtol=1e-6, atol=1e-6 * np.abs(g).max())
        # exact Hessian (not the reference's layout) against differences of the gradient
        H = o.d2psi(model, F0, p, corot_layout_reference=False)
        Hfd = np.stack([fd_grad(lambda v: o.dpsi(model, v.reshape(3, 3, order="F"), p)[i], x0) for i in range(9)])
        assert np.allclose(H, Hfd, rtol=1e-5, atol=1e-5 * np.abs(H).max())
