"""The element math the CUDA kernels use (bartels_gb300/csrc/devmath.cuh),
compiled for the host, against the FP64 oracle: block laws assembled into the
12x12 element Hessian, PSD projection (fast and slow paths), energies,
stresses and the 3x3 SVD, in FP64 (tight) and FP32 (kernel precision)."""
import ctypes as C

import numpy as np
import pytest

from conftest import devmath

D = C.POINTER(C.c_double)
Fp = C.POINTER(C.c_float)
MODEL_ID = {"neohookean": 0, "stvk": 1, "corotational": 2, "neohookean_isochoric": 3, "arap": 4,
            "linear_elasticity": 5}
PARAMS = {"neohookean": np.array([3.5e5, 1.2e6]), "neohookean_isochoric": np.array([3.5e5, 1.2e6]),
          "stvk": np.array([2.4e6, 7e5]), "corotational": np.array([2.4e6, 7e5]), "arap": np.array([9e5, 0.0]),
          "linear_elasticity": np.array([2e6, 0.45])}


def device_params(model, p):
    """The kernels take linear elasticity as the Lame pair (lambda, mu)."""
    if model != "linear_elasticity":
        return p
    E, nu = p
    return np.array([E * nu / ((1 + nu) * (1 - 2 * nu)), E / (2 * (1 + nu))])


def dp(a):
    return a.ctypes.data_as(D)


def fp(a):
    return a.ctypes.data_as(Fp)


def random_tet(rng, amp):
    X = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1.0]]) * 0.1 + 0.02 * rng.standard_normal((4, 3))
    x = X @ (np.eye(3) + amp * rng.standard_normal((3, 3))).T + 0.001 * rng.standard_normal((4, 3))
    return X, x


def oracle_element(oracle, model, X, x, p, psd_tol, exact):
    E = np.array([[0, 1, 2, 3]], np.int32)
    dphi = oracle.dphi_dX(X, E)
    vol = oracle.volume(X, E)
    K = oracle.tetmesh_dq2_elements(model, E, x.ravel(), dphi, vol, p[None, :], psd_tol=psd_tol,
                                    corot_layout_reference=not exact)[0]
    return K, dphi[0], vol[0]


def lib_element(model, x, dphi12, vol, p, psd_tol, exact, dtype):
    L = devmath()
    dphi9 = np.array([dphi12[a + 4 * d] for a in (1, 2, 3) for d in range(3)])
    F = np.zeros(9)
    xs = [np.ascontiguousarray(x[a]) for a in range(4)]
    L.dm_def_grad_d(*[dp(v) for v in xs], dp(dphi9), 0, dp(F))
    pv = vol * device_params(model, p)
    if dtype == np.float64:
        out = np.zeros(144)
        slow = L.dm_element_hessian_d(MODEL_ID[model], dp(F), dp(pv), dp(dphi9), int(exact), int(psd_tol is not None),
                                      C.c_double(psd_tol or 0.0), dp(out))
    else:
        F32, pv32, d32 = (np.ascontiguousarray(a, np.float32) for a in (F, pv, dphi9))
        out = np.zeros(144, np.float32)
        slow = L.dm_element_hessian_f(MODEL_ID[model], fp(F32), fp(pv32), fp(d32), int(exact),
                                      int(psd_tol is not None), C.c_float(psd_tol or 0.0), fp(out))
    return out.reshape(12, 12).astype(np.float64), slow


@pytest.mark.parametrize("model", list(MODEL_ID))
@pytest.mark.parametrize("exact", [False, True])
def test_element_hessian_fp64(oracle, model, exact):
    if exact and model not in ("corotational", "arap"):
        pytest.skip("flag only affects the corotational law")
    rng = np.random.default_rng(11)
    for _ in range(20):
        X, x = random_tet(rng, 0.2)
        K_ref, dphi, vol = oracle_element(oracle, model, X, x, PARAMS[model], None, exact)
        K, _ = lib_element(model, x, dphi, vol, PARAMS[model], None, exact, np.float64)
        assert np.linalg.norm(K - K_ref) <= 1e-10 * np.linalg.norm(K_ref)


@pytest.mark.parametrize("model", list(MODEL_ID))
def test_element_hessian_psd_fp64(oracle, model):
    rng = np.random.default_rng(12)
    slow_seen = fast_seen = 0
    for k in range(40):
        X, x = random_tet(rng, 0.6 if k % 2 else 0.05)
        for tol in (1e-6, 1e-3):
            K_ref, dphi, vol = oracle_element(oracle, model, X, x, PARAMS[model], tol, False)
            K, slow = lib_element(model, x, dphi, vol, PARAMS[model], tol, False, np.float64)
            slow_seen += slow
            fast_seen += 1 - slow
            assert np.linalg.norm(K - K_ref) <= 1e-9 * np.linalg.norm(K_ref)
    # linear elasticity has the 3 infinitesimal rotations in its null space, so
    # simple_psd_fix always changes it (the slow path)
    assert fast_seen > 0 or model == "linear_elasticity"


def test_psd_slow_path_is_exercised(oracle):
    """Strongly compressed Neo-Hookean and StVK elements are indefinite."""
    rng = np.random.default_rng(13)
    seen = 0
    for _ in range(40):
        X, x = random_tet(rng, 0.0)
        x = X @ np.diag([0.5, 1.2, 0.6]) + 0.02 * rng.standard_normal((4, 3))
        for model in ("stvk", "neohookean"):
            K_ref, dphi, vol = oracle_element(oracle, model, X, x, PARAMS[model], 1e-6, False)
            K, slow = lib_element(model, x, dphi, vol, PARAMS[model], 1e-6, False, np.float64)
            seen += slow
            assert np.linalg.norm(K - K_ref) <= 1e-9 * np.linalg.norm(K_ref)
    assert seen > 0


@pytest.mark.parametrize("model", list(MODEL_ID))
def test_element_hessian_fp32(oracle, model):
    rng = np.random.default_rng(14)
    for _ in range(20):
        X, x = random_tet(rng, 0.2)
        for tol in (None, 1e-6):
            K_ref, dphi, vol = oracle_element(oracle, model, X, x, PARAMS[model], tol, False)
            K, _ = lib_element(model, x, dphi, vol, PARAMS[model], tol, False, np.float32)
            assert np.linalg.norm(K - K_ref) <= 2e-5 * np.linalg.norm(K_ref)


@pytest.mark.parametrize("model", list(MODEL_ID))
def test_energy_and_stress_fp64(oracle, model):
    L = devmath()
    rng = np.random.default_rng(15)
    p = PARAMS[model]
    for _ in range(30):
        F = np.eye(3) + 0.2 * rng.standard_normal((3, 3))
        if model.startswith("neo") and np.linalg.det(F) <= 0:
            continue
        fv = np.ascontiguousarray(F.ravel(order="F"))
        pd = np.ascontiguousarray(device_params(model, p))
        e = L.dm_psi_d(MODEL_ID[model], dp(fv), dp(pd))
        e_ref = oracle.psi(model, F, p)
        assert abs(e - e_ref) <= 1e-11 * max(abs(e_ref), 1.0)
        P = np.zeros(9)
        L.dm_pk1_d(MODEL_ID[model], dp(fv), dp(pd), dp(P))
        P_ref = oracle.dpsi(model, F, p)
        assert np.linalg.norm(P - P_ref) <= 1e-11 * np.linalg.norm(P_ref)


def test_svd3_float_and_double(oracle):
    L = devmath()
    rng = np.random.default_rng(16)
    for k in range(100):
        F = rng.standard_normal((3, 3)) if k % 3 == 0 else np.eye(3) + 0.3 * rng.standard_normal((3, 3))
        U0, S0, V0 = oracle.svd3(F)
        fv = np.ascontiguousarray(F.ravel(order="F"))
        U, S, V = np.zeros(9), np.zeros(3), np.zeros(9)
        L.dm_svd3_d(dp(fv), dp(U), dp(S), dp(V))
        assert np.allclose(S, S0, rtol=1e-12, atol=1e-13)
        Um, Vm = U.reshape(3, 3, order="F"), V.reshape(3, 3, order="F")
        assert np.linalg.norm(Um @ np.diag(S) @ Vm.T - F) <= 1e-12 * np.linalg.norm(F)
        f32 = fv.astype(np.float32)
        U32, S32, V32 = np.zeros(9, np.float32), np.zeros(3, np.float32), np.zeros(9, np.float32)
        L.dm_svd3_f(fp(f32), fp(U32), fp(S32), fp(V32))
        assert np.allclose(S32, S0, rtol=2e-5, atol=2e-6 * np.abs(S0).max())
        Um, Vm = U32.reshape(3, 3, order="F").astype(float), V32.reshape(3, 3, order="F").astype(float)
        assert np.linalg.norm(Um @ np.diag(S32.astype(float)) @ Vm.T - F) <= 1e-5 * np.linalg.norm(F)


def test_svd3_double_hard_cases():
    """The FP64 SVD (FP32 warm start, Newton-Schulz re-orthonormalisation, FP64
    sweeps) at machine precision on near-rest, rotated, repeated, nearly
    repeated and inverted deformation gradients."""
    L = devmath()
    rng = np.random.default_rng(17)

    def rot():
        q, _ = np.linalg.qr(rng.standard_normal((3, 3)))
        return q * np.sign(np.linalg.det(q))
    for k in range(100):
        t = k % 5
        if t == 0:
            F = np.eye(3) + 1e-6 * rng.standard_normal((3, 3))
        elif t == 1:
            F = rot()
        elif t == 2:
            F = rot() @ np.diag([1.0, 1.0, 2.0]) @ rot()
        elif t == 3:
            F = rot() @ np.diag([1.5, 0.7, -0.3]) @ rot()
        else:
            F = rot() @ np.diag([1.0, 1.0 + 1e-9, 1.0 - 1e-9]) @ rot()
        fv = np.ascontiguousarray(F.ravel(order="F"))
        U, S, V = np.zeros(9), np.zeros(3), np.zeros(9)
        L.dm_svd3_d(dp(fv), dp(U), dp(S), dp(V))
        Um, Vm = U.reshape(3, 3, order="F"), V.reshape(3, 3, order="F")
        assert np.linalg.norm(Um @ np.diag(S) @ Vm.T - F) <= 1e-14 * np.linalg.norm(F), (k, t)
        assert np.linalg.norm(Vm.T @ Vm - np.eye(3)) <= 1e-14 and np.linalg.norm(Um.T @ Um - np.eye(3)) <= 1e-14
        assert np.linalg.det(Um) > 0 and np.linalg.det(Vm) > 0
        sv = np.sort(np.abs(S))[::-1]
        assert np.abs(sv - np.linalg.svd(F, compute_uv=False)).max() <= 1e-14 * sv[0], (k, t)
        assert (S[2] < 0) == (np.linalg.det(F) < 0)


@pytest.mark.parametrize("model", ["neohookean", "neohookean_isochoric", "stvk"])
def test_cancellation_free_energy_accuracy(oracle, model):
    """psi from the displacement gradient H = F - I (used by the GPU energy and
    line search) against a 40-digit evaluation of the reference's formula: the
    textbook FP64 form loses ~eps/|H|^2 near rest, this one must not."""
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.dps = 40
    L = devmath()
    L.dm_psi_disp_d.restype = C.c_double
    rng = np.random.default_rng(21)
    p = PARAMS[model]
    for scale in (1e-6, 1e-4, 1e-2, 0.2):
        for _ in range(5):
            H = scale * rng.standard_normal((3, 3))
            F = mpmath.matrix([[mpmath.mpf(1) * (i == j) + mpmath.mpf(float(H[i, j])) for j in range(3)]
                               for i in range(3)])
            J = mpmath.det(F)
            I1 = sum(F[i, j] ** 2 for i in range(3) for j in range(3))
            if model == "neohookean":
                ref = p[0] * (I1 - 3 - 2 * mpmath.log(J)) + p[1] * (J - 1) ** 2
            elif model == "neohookean_isochoric":
                ref = p[0] * (J ** (mpmath.mpf(-2) / 3) * I1 - 3) + p[1] * (J - 1) ** 2
            else:
                Em = (F.T * F - mpmath.eye(3)) / 2
                ref = p[1] * sum((Em * Em)[i, i] for i in range(3)) + p[0] / 2 * sum(Em[i, i] for i in range(3)) ** 2
            hv = np.ascontiguousarray(H.ravel(order="F"))
            got = L.dm_psi_disp_d(MODEL_ID[model], dp(hv), dp(p))
            assert abs(got - float(ref)) <= 1e-13 * abs(float(ref)), (scale, got, float(ref))


@pytest.mark.parametrize("model", ["neohookean", "stvk", "corotational"])
def test_fp32_rest_and_rigid_elements_take_the_fast_path(oracle, model):
    """At rest or after a rigid rotation the three rotation modes have
    eigenvalue zero up to FP32 rounding; the FP32 fast test accepts them
    (within the FP32 eigen-solver's own rounding) and the result matches the
    exactly projected matrix. A strained element (1e-3) still takes the slow
    path."""
    rng = np.random.default_rng(17)
    for k in range(10):
        X, _ = random_tet(rng, 0.0)
        A = rng.standard_normal((3, 3))
        Q, _ = np.linalg.qr(A)
        Q *= np.sign(np.linalg.det(Q))
        x = X if k % 2 == 0 else X @ Q.T + rng.standard_normal(3)
        K_ref, dphi, vol = oracle_element(oracle, model, X, x, PARAMS[model], 1e-6, False)
        K, slow = lib_element(model, x, dphi, vol, PARAMS[model], 1e-6, False, np.float32)
        assert slow == 0
        assert np.linalg.norm(K - K_ref) <= 2e-5 * np.linalg.norm(K_ref)
    X, _ = random_tet(rng, 0.0)
    x = X @ np.diag([1.0, 1.0, 0.999])  # compressed along z: negative rotation eigenvalues
    K_ref, dphi, vol = oracle_element(oracle, model, X, x, PARAMS[model], 1e-6, False)
    K, slow = lib_element(model, x, dphi, vol, PARAMS[model], 1e-6, False, np.float32)
    assert slow == 1 or model == "stvk"
    assert np.linalg.norm(K - K_ref) <= 2e-5 * np.linalg.norm(K_ref)


@pytest.mark.parametrize("model", ["neohookean", "neohookean_isochoric", "stvk", "corotational", "arap"])
def test_known_answers_rest_and_rigid_rotations(oracle, model):
    """psi = 0 and dpsi/dF = 0 at F = I and at any rotation F = R, for every
    hyperelastic law, in the library's math (FP64, on the host) and the oracle."""
    L = devmath()
    p = PARAMS[model]
    rng = np.random.default_rng(21)
    rots = [np.eye(3)]
    for _ in range(5):
        Q, _ = np.linalg.qr(rng.standard_normal((3, 3)))
        rots.append(Q * np.sign(np.linalg.det(Q)))  # proper rotation
    scale = np.abs(p).max()
    for R in rots:
        fv = np.ascontiguousarray(R.ravel(order="F"))
        pd = np.ascontiguousarray(p, np.float64)
        e = L.dm_psi_d(MODEL_ID[model], dp(fv), dp(pd))
        P = np.zeros(9)
        L.dm_pk1_d(MODEL_ID[model], dp(fv), dp(pd), dp(P))
        assert abs(e) <= 1e-12 * scale and np.abs(P).max() <= 1e-9 * scale, (model, e, np.abs(P).max())
        assert abs(oracle.psi(model, R, p)) <= 1e-12 * scale
        assert np.abs(oracle.dpsi(model, R, p)).max() <= 1e-9 * scale
