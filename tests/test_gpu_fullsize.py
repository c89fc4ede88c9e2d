"""Parity at the benchmark's size: the n = 96 Kuhn cube (912,673 vertices,
5,308,416 tets, 121,188,969 Hessian entries) through the C ABI.

The oracle cannot assemble the whole Hessian in seconds, so two kinds of check:
  * exact rows: every tet incident to 500 random vertices goes through the
    oracle, which gives those vertices' complete Hessian rows and gradient
    entries; the GPU's rows must have the same columns (bit-exact) and values
    within 1e-5 of the largest entry (FP32 Hessian; within 1e-4 of each row's
    own largest entry), the gradient within 1e-10 (FP64). The energy is
    compared over all tets (FP64, 1e-10).
  * size-independent properties of the whole result: the closed-form entry
    count and a symmetric pattern, H t = 0 for rigid translations t, rotation
    invariance of the energy and equivariance of the gradient, and H v against
    central differences of the FP64 gradient.
"""
import numpy as np
import pytest
import scipy.sparse as sp

import bartels_gb300 as bg
from bartels_gb300.meshes import cube_counts, kuhn_cube, material_params

pytestmark = pytest.mark.gpu

N = 96


@pytest.fixture(scope="module")
def mesh(oracle):
    V, E = kuhn_cube(N)
    dphi, vol = oracle.dphi_dX(V, E), oracle.volume(V, E)
    plan = bg.MeshPlan(V, E)
    yield V, E, dphi, vol, plan
    plan.close()


def deformed(V, stretch, amp, seed):
    rng = np.random.default_rng(seed)
    return (V * np.asarray(stretch) + rng.uniform(-amp / N, amp / N, V.shape)).ravel()


def sample_vertices(nV, seed, count=500):
    rng = np.random.default_rng(seed)
    return np.sort(rng.choice(nV, size=count, replace=False))


def check_rows(oracle, model, V, E, q, dphi, vol, params, psd_tol, H, g, verts):
    """The GPU's Hessian rows / gradient entries of `verts` against the oracle
    on the tets incident to them (which make those rows complete)."""
    inc = np.isin(E, verts).any(axis=1)
    args = (len(V), E[inc], q, dphi[inc], vol[inc], params[inc])
    Hs = oracle.tetmesh_dq2(model, *args, psd_tol=psd_tol)
    gs = oracle.tetmesh_dq(model, *args)
    rows = (3 * verts[:, None] + np.arange(3)).ravel()
    err = big = row_rel = 0.0
    for r in rows:
        a0, a1 = H.indptr[r], H.indptr[r + 1]
        b0, b1 = Hs.indptr[r], Hs.indptr[r + 1]
        assert np.array_equal(H.indices[a0:a1], Hs.indices[b0:b1]), r
        ref = Hs.data[b0:b1]
        d = np.abs(H.data[a0:a1] - ref).max()
        err, big = max(err, d), max(big, np.abs(ref).max())
        row_rel = max(row_rel, d / np.abs(ref).max())
    # relative to the largest entry, and per row relative to the row's own largest entry
    assert err <= 1e-5 * big, err / big
    assert row_rel <= 1e-5, row_rel
    assert np.linalg.norm(g[rows] - gs[rows]) <= 1e-10 * np.linalg.norm(gs[rows])
    return err / big


def test_pattern_counts_and_symmetry(mesh):
    V, E, _, _, plan = mesh
    c = cube_counts(N)
    assert (plan.n, plan.nnz) == (c["ndof"], c["nnz"])
    if N == 96:
        assert (c["ndof"], c["nnz"]) == (3 * 912673, 121188969)
    rp, ci = plan.pattern()
    assert np.all(np.diff(rp) > 0)
    # block pattern: the columns 3j of the scalar rows 3v
    row = np.repeat(np.arange(plan.n, dtype=np.int32), np.diff(rp))
    keep = (row % 3 == 0) & (ci % 3 == 0)
    brow, bcol = row[keep] // 3, ci[keep] // 3
    del row, keep
    assert len(brow) == c["nnz"] // 9
    B = sp.csr_matrix((np.ones(len(brow), np.int8), (brow, bcol)), shape=(len(V), len(V)))
    assert (B != B.T).nnz == 0
    assert np.all(B.diagonal() == 1)


@pytest.mark.parametrize("model, stretch, amp, psd_tol, seed", [
    ("neohookean", (1.1, 0.9, 1.0), 0.02, 1e-6, 1),
    ("stvk", (1.0, 1.0, 0.6), 0.2, 1e-6, 2),          # compressed: many indefinite elements, projected
    ("corotational", (1.05, 0.95, 1.1), 0.1, None, 3),
])
def test_sampled_rows_energy_and_gradient(oracle, mesh, model, stretch, amp, psd_tol, seed):
    V, E, dphi, vol, plan = mesh
    params = material_params(model, len(E), 2e6, 0.45)
    q = deformed(V, stretch, amp, seed)
    plan.set_element_data(dphidX=dphi, volume=vol, params=params)
    H = plan.dq2(model, q, psd_tol=psd_tol)
    g = plan.dq(model, q)
    check_rows(oracle, model, V, E, q, dphi, vol, params, psd_tol, H, g, sample_vertices(len(V), 7))
    del H
    e = plan.q(model, q)
    e_ref = oracle.tetmesh_q(model, E, q, dphi, vol, params)
    assert abs(e - e_ref) <= 1e-10 * abs(e_ref)


def test_translation_rotation_and_finite_differences(mesh):
    V, E, dphi, vol, plan = mesh
    model = "neohookean"
    params = material_params(model, len(E), 2e6, 0.45)
    plan.set_element_data(dphidX=dphi, volume=vol, params=params)
    q = deformed(V, (1.1, 0.9, 1.0), 0.05, seed=3)
    H = plan.dq2(model, q)
    # rigid translations are in the null space of the unprojected Hessian
    rowabs = np.asarray(abs(H).sum(axis=1)).ravel()
    for d in range(3):
        t = np.zeros(3 * len(V))
        t[d::3] = 1.0
        assert np.abs(H @ t).max() <= 1e-5 * rowabs.max()
    # H v against central differences of the FP64 gradient
    rng = np.random.default_rng(4)
    v = rng.standard_normal(3 * len(V)) / N
    eps = 1e-3
    fd = (plan.dq(model, q + eps * v) - plan.dq(model, q - eps * v)) / (2 * eps)
    assert np.linalg.norm(H @ v - fd) <= 1e-5 * np.linalg.norm(fd)
    del H
    # rotation: energy invariant, gradient rotates with the mesh
    ax = np.array([1.0, 2.0, 3.0]) / np.sqrt(14.0)
    K = np.array([[0, -ax[2], ax[1]], [ax[2], 0, -ax[0]], [-ax[1], ax[0], 0]])
    R = np.eye(3) + np.sin(0.7) * K + (1 - np.cos(0.7)) * K @ K
    qr = (q.reshape(-1, 3) @ R.T).ravel()
    e, er = plan.q(model, q), plan.q(model, qr)
    assert abs(er - e) <= 1e-11 * abs(e)
    g, gr = plan.dq(model, q), plan.dq(model, qr)
    assert np.linalg.norm(gr - (g.reshape(-1, 3) @ R.T).ravel()) <= 1e-10 * np.linalg.norm(g)
