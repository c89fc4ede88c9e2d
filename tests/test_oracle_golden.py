"""Pin the FP64 oracle against every golden vector the reference's tests hold.

tests/test_constitutive_model.cpp (F known answer, NH Hessian of coarser_bunny),
tests/test_assemble.cpp (mass matrix, force = M g), tests/test_flatten_multiply.cpp
(vec identities).
"""
import numpy as np
import scipy.sparse as sp

from conftest import load_golden_csr, load_golden_mesh

YM, NU = 6e5, 0.4  # tests/test_constitutive_model.cpp:73-76


def bunny_setup(o):
    V, E = load_golden_mesh("coarser_bunny")
    dphi = o.dphi_dX(V, E)
    vol = o.volume(V, E)
    q = (V * np.array([2.0, 4.0, 3.0])).ravel()
    D = 0.5 * (YM * NU) / ((1.0 + NU) * (1.0 - 2.0 * NU))
    Cc = 0.5 * YM / (2.0 * (1.0 + NU))
    params = np.tile([Cc, D], (len(E), 1))
    return V, E, dphi, vol, q, params


def test_deformation_gradient_known_answer(oracle):
    V, E, dphi, vol, q, params = bunny_setup(oracle)
    target = np.array([2, 0, 0, 0, 4, 0, 0, 0, 3.0])
    for t in range(len(E)):
        B = oracle.build_B(dphi[t])
        qe = np.concatenate([q[3 * E[t, a]:3 * E[t, a] + 3] for a in range(4)])
        assert np.linalg.norm(B @ qe - target) < 1e-8


def test_flatten_multiply_identity(oracle):
    rng = np.random.default_rng(1)
    for _ in range(20):
        dphi = rng.standard_normal((4, 3))
        A = rng.standard_normal((3, 4))
        B = oracle.build_B(dphi.ravel(order="F"))
        assert np.linalg.norm(B @ A.ravel(order="F") - (A @ dphi).ravel(order="F")) < 1e-12


def test_volumes_positive(oracle):
    V, E, dphi, vol, q, params = bunny_setup(oracle)
    assert vol.min() > 0


def test_golden_patterns(oracle):
    V, E, dphi, vol, q, params = bunny_setup(oracle)
    H_ref = load_golden_csr("H_neohookean_coarser_bunny")
    M_ref = load_golden_csr("M_coarse_bunny")
    H = oracle.tetmesh_dq2("neohookean", len(V), E, q, dphi, vol, params)
    M = oracle.mass_matrix(len(V), E, np.full(len(E), 0.1), vol)
    for A, R in ((H, H_ref), (M, M_ref)):
        assert np.array_equal(A.indptr, R.indptr) and np.array_equal(A.indices, R.indices)
    V2, E2 = load_golden_mesh("two_tets")
    M2 = oracle.mass_matrix(len(V2), E2, np.ones(len(E2)), oracle.volume(V2, E2))
    R2 = load_golden_csr("M_two_tets")
    assert np.array_equal(M2.indptr, R2.indptr) and np.array_equal(M2.indices, R2.indices)


def test_golden_hessian_isochoric_law(oracle):
    """data/matrices/H_neohookean_coarser_bunny.txt matches the isochoric law to
    the reference's own criterion ||H - H_ref|| / H(0,0) < 1e-8."""
    V, E, dphi, vol, q, params = bunny_setup(oracle)
    H_ref = load_golden_csr("H_neohookean_coarser_bunny")
    H = oracle.tetmesh_dq2("neohookean_isochoric", len(V), E, q, dphi, vol, params)
    assert sp.linalg.norm(H - H_ref) / H[0, 0] < 1e-8


def test_golden_hessian_is_not_the_current_law(oracle):
    """The current ln(J) law (src/d2psi_neohookean_dF2.cpp:185-283) does not
    reproduce the golden file: the reference's own test would print FAILED."""
    V, E, dphi, vol, q, params = bunny_setup(oracle)
    H_ref = load_golden_csr("H_neohookean_coarser_bunny")
    H = oracle.tetmesh_dq2("neohookean", len(V), E, q, dphi, vol, params)
    assert sp.linalg.norm(H - H_ref) / H[0, 0] > 0.1


def test_golden_mass_matrix(oracle):
    V, E, dphi, vol, q, params = bunny_setup(oracle)
    M_ref = load_golden_csr("M_coarse_bunny")
    M = oracle.mass_matrix(len(V), E, np.full(len(E), 0.1), vol)
    assert sp.linalg.norm(M - M_ref) < 1e-8


def test_force_is_mass_times_gravity(oracle):
    V, E, dphi, vol, q, params = bunny_setup(oracle)
    g = np.array([0, -9.8, 0])
    M = oracle.mass_matrix(len(V), E, np.full(len(E), 0.1), vol)
    f = oracle.const_ext_force(len(V), E, vol, 0.1 * g)
    assert np.linalg.norm(f - M @ np.tile(g, len(V))) < 1e-8
