"""FP64 CPU restatement of the reference's planar triangle-mesh routines
(linear_tri2d_* / linear_tri2dmesh_*). TEST INFRASTRUCTURE: only tests/ may use it.

It follows the reference's construction literally: the element's 3x3
deformation gradient F = unflatten(B qe + one) with B = flatten_multiply_right(
[dphidX | 0]) P (src/linear_tri2d_neohookean_q.cpp:9-14: P picks the in-plane
entries of the three vertices, `one` sets F33 = 1), energy psi(F) * area,
gradient B^T dpsi(F) * area, Hessian B^T d2psi(F) B * area, with the 3D laws of
the FP64 C++ restatement (oracle/oracle.py). Linear elasticity follows
src/linear_tri2d_linear_elasticity_dq2.cpp:9-44 (strain matrix P2 B, Voigt C of
src/d2psi_linear_elasticity_de2.cpp:8-27). Assembly follows src/assemble.cpp:
element matrices as triplets, duplicates summed (scipy), CSR of the symmetric
pattern.

Parity pins: the reference ships no golden data for triangles; its only 2D test
(tests/test_constitutive_model.cpp:107-135, the corotational gradient of one
triangle at rest, printed) gives the known answer 0, and finite differences tie
energy, gradient and Hessian together (tests/test_tri2d_oracle.py).
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp

from . import oracle as O

# rows of vec(X) (3x3 positions, column-major) picked from the 6 element DOFs
_P = np.zeros((9, 6))
for _a in range(3):
    _P[3 * _a, 2 * _a] = 1.0
    _P[3 * _a + 1, 2 * _a + 1] = 1.0


def dphi_dX(V, E):
    """src/linear_tri2d_dphi_dX.cpp:10-16: rows 1, 2 = inverse22 of [x1-x0, x2-x0],
    row 0 = -(row 1 + row 2); returned (nT, 6) as the column-major flatten of 3x2."""
    V = np.asarray(V, np.float64)
    out = np.zeros((len(E), 6))
    for t, e in enumerate(np.asarray(E)):
        D = np.stack([V[e[1]] - V[e[0]], V[e[2]] - V[e[0]]], axis=1)  # columns = edges
        det = D[0, 0] * D[1, 1] - D[0, 1] * D[1, 0]
        inv = np.array([[D[1, 1], -D[0, 1]], [-D[1, 0], D[0, 0]]]) / det
        d = np.zeros((3, 2))
        d[1:] = inv
        d[0] = -inv.sum(axis=0)
        out[t] = d.ravel(order="F")
    return out


def area(V, E):
    V = np.asarray(V, np.float64)
    out = np.zeros(len(E))
    for t, e in enumerate(np.asarray(E)):
        a, b = V[e[1]] - V[e[0]], V[e[2]] - V[e[0]]
        out[t] = 0.5 * abs(a[0] * b[1] - a[1] * b[0])
    return out


def _B(dphi6):
    """flatten_multiply_right([dphidX | 0]) P: vec(F) = B qe + one (9 x 6)."""
    M = np.zeros((3, 3))
    M[:, :2] = np.asarray(dphi6).reshape(3, 2, order="F")
    # vec(X M) = (M^T kron I3) vec(X)
    return np.kron(M.T, np.eye(3)) @ _P


def _qe(q, e):
    q = np.asarray(q, np.float64)
    return np.concatenate([q[2 * e[0]:2 * e[0] + 2], q[2 * e[1]:2 * e[1] + 2], q[2 * e[2]:2 * e[2] + 2]])


def _F(q, e, dphi6):
    one = np.zeros(9)
    one[8] = 1.0
    return (_B(dphi6) @ _qe(q, e) + one).reshape(3, 3, order="F")


def q_elements(model, E, q, dphidX, area_, params):
    E = np.asarray(E)
    return np.array([O.psi(model, _F(q, e, dphidX[t]), params[t]) * area_[t] for t, e in enumerate(E)])


def energy(model, E, q, dphidX, area_, params):
    return float(np.sum(q_elements(model, E, q, dphidX, area_, params)))


def gradient(model, nV, E, q, dphidX, area_, params):
    g = np.zeros(2 * nV)
    for t, e in enumerate(np.asarray(E)):
        ge = _B(dphidX[t]).T @ O.dpsi(model, _F(q, e, dphidX[t]), params[t]) * area_[t]
        for a in range(3):
            g[2 * e[a]:2 * e[a] + 2] += ge[2 * a:2 * a + 2]
    return g


def _le_hessian(dphi6, params, area_t):
    """src/linear_tri2d_linear_elasticity_dq2.cpp:12-44, C of
    src/d2psi_linear_elasticity_de2.cpp:8-27 with (Young's modulus, Poisson ratio)."""
    P2 = np.zeros((6, 9))
    P2[0, 0] = 1
    P2[1, 4] = 1
    P2[2, 8] = 1
    P2[3, 5] = P2[3, 7] = 1
    P2[4, 2] = P2[4, 6] = 1
    P2[5, 1] = P2[5, 3] = 1
    YM, nu = params
    Cm = np.zeros((6, 6))
    Cm[:3, :3] = nu
    np.fill_diagonal(Cm[:3, :3], 1.0 - nu)
    Cm[3, 3] = Cm[4, 4] = Cm[5, 5] = 0.5 * (1.0 - 2.0 * nu)
    Cm *= YM / ((1.0 + nu) * (1.0 - 2.0 * nu))
    B = P2 @ _B(dphi6)
    return B.T @ Cm @ B * area_t


def hessian_elements(model, E, q, dphidX, area_, params, psd_tol=None, corot_layout_reference=True):
    """corot_layout_reference: the reference's d2psi_stretch_dF2 storage (the
    Hessian at F^T, src/d2psi_stretch_dF2.cpp:37-45); False gives the exact one."""
    out = []
    for t, e in enumerate(np.asarray(E)):
        if model == "linear_elasticity":
            K = _le_hessian(dphidX[t], params[t], area_[t])
        else:
            B = _B(dphidX[t])
            H9 = O.d2psi(model, _F(q, e, dphidX[t]), params[t], corot_layout_reference)
            K = B.T @ H9 @ B * area_[t]
        if psd_tol is not None:
            K = O.psd_fix(K, psd_tol)
        out.append(K)
    return np.array(out)


def assemble(nV, E, Ke):
    """src/assemble.cpp:57-94: triplets of every element matrix, duplicates summed."""
    rows, cols, vals = [], [], []
    for t, e in enumerate(np.asarray(E)):
        dof = np.array([[2 * v, 2 * v + 1] for v in e]).ravel()
        for c in range(6):
            for r in range(6):
                rows.append(dof[r])
                cols.append(dof[c])
                vals.append(Ke[t][r, c])
    H = sp.coo_matrix((vals, (rows, cols)), shape=(2 * nV, 2 * nV)).tocsr()
    H.sum_duplicates()
    H.sort_indices()
    return H


def hessian(model, nV, E, q, dphidX, area_, params, psd_tol=None, corot_layout_reference=True):
    return assemble(nV, E, hessian_elements(model, E, q, dphidX, area_, params, psd_tol, corot_layout_reference))


def mass_matrix(nV, E, density, area_):
    """src/linear_tri2d_mass_matrix.cpp:10-32: density * area * (1/6 diag, 1/12 off) x I2."""
    Ke = []
    for t in range(len(E)):
        m = density[t] * area_[t]
        K = np.kron(np.full((3, 3), m / 12.0) + np.eye(3) * (m / 6.0 - m / 12.0), np.eye(2))
        Ke.append(K)
    return assemble(nV, E, np.array(Ke))


def square_mesh(n, seed=0, jitter=0.0):
    """Unit square split into 2 n^2 triangles (alternating diagonals), vertex
    jitter in units of the cell size."""
    rng = np.random.default_rng(seed)
    xs = np.linspace(0.0, 1.0, n + 1)
    V = np.array([[x, y] for y in xs for x in xs])
    if jitter:
        V[:, :] += jitter / n * rng.uniform(-1, 1, V.shape)
    E = []
    for j in range(n):
        for i in range(n):
            a, b, c, d = j * (n + 1) + i, j * (n + 1) + i + 1, (j + 1) * (n + 1) + i, (j + 1) * (n + 1) + i + 1
            if (i + j) % 2 == 0:
                E += [[a, b, d], [a, d, c]]
            else:
                E += [[a, b, c], [b, d, c]]
    return V, np.array(E, np.int32)


# ------------------------------------------------------------ triangles in space
def dphi_dX_3d(V, E):
    """src/linear_tri3d_dphi_dX.cpp:10-16: T = [x1-x0, x2-x0] (3x2), rows 1, 2 =
    (T^T T)^-1 T^T, row 0 = -(row 1 + row 2); (nT, 9) column-major flatten of 3x3."""
    V = np.asarray(V, np.float64)
    out = np.zeros((len(E), 9))
    for t, e in enumerate(np.asarray(E)):
        Tm = np.stack([V[e[1]] - V[e[0]], V[e[2]] - V[e[0]]], axis=1)
        d = np.zeros((3, 3))
        d[1:] = np.linalg.inv(Tm.T @ Tm) @ Tm.T
        d[0] = -d[1:].sum(axis=0)
        out[t] = d.ravel(order="F")
    return out


def area_3d(V, E):
    V = np.asarray(V, np.float64)
    E = np.asarray(E)
    return 0.5 * np.linalg.norm(np.cross(V[E[:, 1]] - V[E[:, 0]], V[E[:, 2]] - V[E[:, 0]]), axis=1)


def stvk_hessian_3d_elements(E, q, dphidX, N, n, dndq, area_, params, psd_tol=None):
    """src/linear_tri3d_stvk_dq2.cpp:15-42, literally: B = flatten_multiply_right(dphidX)
    + flatten_multiply_right(N) unflatten<3,9>(dndq), F = unflatten(B qe + vec(n N)),
    K = B^T d2psi_stvk(F) B * area."""
    q = np.asarray(q, np.float64)
    out = []
    for t, e in enumerate(np.asarray(E)):
        qe = np.concatenate([q[3 * v:3 * v + 3] for v in e])
        M = np.asarray(dphidX[t]).reshape(3, 3, order="F")
        Na = np.asarray(N[t]).reshape(1, 3)
        fmr_N = np.kron(Na.reshape(3, 1), np.eye(3))  # vec(y Na) = fmr_N y
        B = np.kron(M.T, np.eye(3)) + fmr_N @ np.asarray(dndq[t]).reshape(3, 9, order="F")
        F = (B @ qe + fmr_N @ np.asarray(n[t])).reshape(3, 3, order="F")
        K = B.T @ O.d2psi("stvk", F, params[t]) @ B * area_[t]
        if psd_tol is not None:
            K = O.psd_fix(K, psd_tol)
        out.append(K)
    return np.array(out)


def assemble_3(nV, E, Ke):
    """src/assemble.cpp:57-94 with 3 DOFs per vertex."""
    rows, cols, vals = [], [], []
    for t, e in enumerate(np.asarray(E)):
        dof = np.array([[3 * v, 3 * v + 1, 3 * v + 2] for v in e]).ravel()
        for c in range(9):
            for r in range(9):
                rows.append(dof[r])
                cols.append(dof[c])
                vals.append(Ke[t][r, c])
    H = sp.coo_matrix((vals, (rows, cols)), shape=(3 * nV, 3 * nV)).tocsr()
    H.sum_duplicates()
    H.sort_indices()
    return H


def stvk_hessian_3d(nV, E, q, dphidX, N, n, dndq, area_, params, psd_tol=None):
    return assemble_3(nV, E, stvk_hessian_3d_elements(E, q, dphidX, N, n, dndq, area_, params, psd_tol))
