"""Pointwise laws on the GPU (bartels_pointwise_laws; the reference's
psi_<law>_F, dpsi_<law>_dF, d2psi_<law>_dF2) against the FP64 oracle, their
consistency under central differences, and the MATLAB gateways
dpsi_neohookean_dF / d2psi_neohookean_dF2 / d2psi_stvk_dF2 in MATLAB's layout."""
import numpy as np
import pytest
import scipy.sparse as sp

import bartels_gb300 as bg
from bartels_gb300 import mex
from bartels_gb300.meshes import material_params

pytestmark = pytest.mark.gpu

ORACLE_MODELS = ["neohookean", "neohookean_isochoric", "stvk", "corotational", "arap"]


def random_F(n, seed, spread):
    rng = np.random.default_rng(seed)
    F = np.eye(3) + spread * rng.standard_normal((n, 3, 3))
    F[np.linalg.det(F) < 0.2] = np.eye(3)  # keep J well away from 0 for the log / inverse laws
    return F


@pytest.mark.parametrize("model", ORACLE_MODELS)
def test_laws_match_oracle(oracle, model):
    F = random_F(300, 1, 0.25)
    p = material_params(model, len(F), 2e6, 0.45)
    psi, dpsi, d2 = bg.pointwise_laws(model, F, p)
    assert psi.shape == (300,) and dpsi.shape == (300, 9) and d2.shape == (300, 9, 9)
    tol = 1e-9 if model in ("corotational", "arap") else 1e-11
    for t in range(len(F)):
        e = oracle.psi(model, F[t], p[t])
        assert abs(psi[t] - e) <= tol * (abs(e) + p[t].max()), (t, psi[t], e)
        g = oracle.dpsi(model, F[t], p[t])
        assert np.abs(dpsi[t] - g).max() <= tol * np.abs(g).max() + 1e-9 * p[t].max(), t
        H = oracle.d2psi(model, F[t], p[t])
        assert np.abs(d2[t] - H).max() <= tol * np.abs(H).max(), t


@pytest.mark.parametrize("model", ["neohookean", "neohookean_isochoric", "stvk", "linear_elasticity"])
def test_laws_are_consistent_under_central_differences(model):
    F = random_F(40, 2, 0.2)
    p = material_params(model, len(F), 1e6, 0.4)
    psi, dpsi, d2 = bg.pointwise_laws(model, F, p)
    h = 1e-6
    for r in range(9):
        E = np.zeros(9)
        E[r] = h
        dF = E.reshape(3, 3, order="F")  # column-major flatten position r
        pp, gp, _ = bg.pointwise_laws(model, F + dF, p, d2psi=False)
        pm, gm, _ = bg.pointwise_laws(model, F - dF, p, d2psi=False)
        assert np.abs((pp - pm) / (2 * h) - dpsi[:, r]).max() <= 1e-6 * np.abs(dpsi).max()
        assert np.abs((gp - gm) / (2 * h) - d2[:, :, r]).max() <= 1e-6 * np.abs(d2).max()
    assert np.abs(d2 - d2.transpose(0, 2, 1)).max() <= 1e-12 * np.abs(d2).max()


def test_single_F_and_named_drop_ins(oracle):
    F = random_F(1, 3, 0.2)[0]
    p = material_params("stvk", 1, 2e6, 0.45)[0]
    assert np.isclose(bg.psi_stvk_F(F, p), oracle.psi("stvk", F, p), rtol=1e-12)
    assert np.allclose(bg.dpsi_stvk_dF(F, p), oracle.dpsi("stvk", F, p), rtol=1e-11, atol=0)
    q = material_params("neohookean", 1, 2e6, 0.45)[0]
    H = bg.d2psi_neohookean_dF2(F, q)
    assert H.shape == (9, 9) and np.allclose(H, oracle.d2psi("neohookean", F, q), rtol=1e-11, atol=1e-6)
    # (n, 9) rows of column-major flattens are accepted as well
    Fb = random_F(5, 4, 0.2)
    flat = Fb.transpose(0, 2, 1).reshape(5, 9)
    assert np.array_equal(bg.pointwise_laws("stvk", flat, np.tile(p, (5, 1)))[1],
                          bg.pointwise_laws("stvk", Fb, np.tile(p, (5, 1)))[1])


@pytest.mark.parametrize("routine, model", [("d2psi_neohookean_dF2", "neohookean"), ("d2psi_stvk_dF2", "stvk")])
def test_hessian_gateways_block_diagonal(oracle, routine, model):
    F = random_F(7, 5, 0.2)
    p = material_params(model, 7, 2e6, 0.45)
    flat = F.transpose(0, 2, 1).reshape(7, 9)   # MATLAB: F(t, :) = [F11 F21 F31 F12 ...]
    E = np.arange(28, dtype=float).reshape(7, 4) + 1
    H = mex.call(routine, E, flat, p)
    assert isinstance(H, sp.csc_matrix) and H.shape == (63, 63) and H.nnz == 7 * 81
    ref = sp.block_diag([sp.coo_matrix(oracle.d2psi(model, F[t], p[t])) for t in range(7)], format="csc")
    assert np.array_equal(H.indptr, ref.indptr) and np.array_equal(H.indices, ref.indices)
    assert np.abs(H.data - ref.data).max() <= 1e-11 * np.abs(ref.data).max()


def test_gradient_gateway(oracle):
    F = random_F(6, 6, 0.2)
    p = material_params("neohookean", 6, 2e6, 0.45)
    g = mex.call("dpsi_neohookean_dF", np.ones((6, 4)), F.transpose(0, 2, 1).reshape(6, 9), p)
    assert g.shape == (54, 1)
    ref = np.concatenate([oracle.dpsi("neohookean", F[t], p[t]) for t in range(6)])
    assert np.abs(g[:, 0] - ref).max() <= 1e-11 * np.abs(ref).max()
