"""Property-based checks of the element laws on deformation gradients drawn
by hypothesis (J >= 0.2, entries within 0.6 of the identity): the kernels'
math compiled for the host (devmath.cuh) equals the FP64 oracle, and the
oracle's gradient and Hessian equal centred differences of its energy and
gradient (the reference's scheme, src/finite_differences.cpp:42-80)."""
import numpy as np
import pytest

hyp = pytest.importorskip("hypothesis")
st = pytest.importorskip("hypothesis.strategies")
from hypothesis import given, settings, assume, HealthCheck  # noqa: E402

from conftest import devmath  # noqa: E402
from test_devmath_cpu import MODEL_ID, PARAMS, dp  # noqa: E402

LAWS = ["neohookean", "neohookean_isochoric", "stvk", "corotational", "arap"]
F_ENTRIES = st.lists(st.floats(-0.6, 0.6, allow_nan=False, allow_infinity=False), min_size=9, max_size=9)


def as_F(entries):
    return np.eye(3) + np.array(entries).reshape(3, 3)


@pytest.mark.parametrize("model", LAWS)
@settings(max_examples=60, deadline=None, derandomize=True, suppress_health_check=[HealthCheck.function_scoped_fixture])
@given(entries=F_ENTRIES)
def test_library_laws_equal_the_oracle(oracle, model, entries):
    F = as_F(entries)
    assume(np.linalg.det(F) >= 0.2)
    if model in ("corotational", "arap"):
        s = np.linalg.svd(F, compute_uv=False)
        assume(np.min(np.abs(np.diff(np.sort(s)))) > 1e-3)  # away from the repeated-value branch
    L = devmath()
    p = PARAMS[model]
    fv = np.ascontiguousarray(F.ravel(order="F"))
    pd = np.ascontiguousarray(p, np.float64)
    e = L.dm_psi_d(MODEL_ID[model], dp(fv), dp(pd))
    P = np.zeros(9)
    L.dm_pk1_d(MODEL_ID[model], dp(fv), dp(pd), dp(P))
    e_ref, P_ref = oracle.psi(model, F, p), oracle.dpsi(model, F, p)
    scale = np.abs(p).max()
    assert abs(e - e_ref) <= 1e-10 * (abs(e_ref) + scale)
    assert np.abs(P - P_ref).max() <= 1e-9 * (np.abs(P_ref).max() + scale)


@pytest.mark.parametrize("model", ["neohookean", "neohookean_isochoric", "stvk"])
@settings(max_examples=40, deadline=None, derandomize=True, suppress_health_check=[HealthCheck.function_scoped_fixture])
@given(entries=F_ENTRIES)
def test_oracle_derivatives_are_centred_differences(oracle, model, entries):
    F = as_F(entries)
    assume(np.linalg.det(F) >= 0.2)
    p = PARAMS[model]
    P = oracle.dpsi(model, F, p)
    H = oracle.d2psi(model, F, p)
    h = 1e-6
    for r in range(9):
        dF = np.zeros(9)
        dF[r] = h
        D = dF.reshape(3, 3, order="F")
        fd = (oracle.psi(model, F + D, p) - oracle.psi(model, F - D, p)) / (2 * h)
        assert abs(fd - P[r]) <= 1e-5 * (np.abs(P).max() + np.abs(p).max())
        gd = (oracle.dpsi(model, F + D, p) - oracle.dpsi(model, F - D, p)) / (2 * h)
        assert np.abs(gd - H[:, r]).max() <= 1e-5 * (np.abs(H).max() + np.abs(p).max())


def _element(model, F, psd, dtype):
    import ctypes as C
    L = devmath()
    dphi9 = np.array([1.0, 0.1, -0.2, 0.05, 1.1, 0.0, -0.1, 0.2, 0.9])
    pv = PARAMS[model] * (1.0 / 6.0)
    fv = np.ascontiguousarray(F.ravel(order="F"))
    if dtype == np.float64:
        out = np.zeros(144)
        L.dm_element_hessian_d(MODEL_ID[model], dp(fv), dp(np.ascontiguousarray(pv)), dp(dphi9), 0, int(psd),
                               C.c_double(1e-6), dp(out))
    else:
        Fp = C.POINTER(C.c_float)
        f32, p32, d32 = (np.ascontiguousarray(a, np.float32) for a in (fv, pv, dphi9))
        out = np.zeros(144, np.float32)
        L.dm_element_hessian_f(MODEL_ID[model], f32.ctypes.data_as(Fp), p32.ctypes.data_as(Fp),
                               d32.ctypes.data_as(Fp), 0, int(psd), C.c_float(1e-6), out.ctypes.data_as(Fp))
    return out.astype(np.float64)


@pytest.mark.parametrize("model", ["neohookean", "stvk", "corotational"])
@pytest.mark.parametrize("psd", [0, 1])
@settings(max_examples=60, deadline=None, derandomize=True)
@given(entries=F_ENTRIES)
def test_fp32_element_hessian_within_the_kernel_bound(model, psd, entries):
    """The FP32 element Hessian the kernels assemble stays within 1e-5 of the
    largest entry of the FP64 one (projected or not)."""
    F = as_F(entries)
    assume(np.linalg.det(F) >= 0.2)
    if model == "corotational":
        s = np.linalg.svd(F, compute_uv=False)
        assume(np.min(np.abs(np.diff(np.sort(s)))) > 1e-3)
    K64 = _element(model, F, psd, np.float64)
    K32 = _element(model, F, psd, np.float32)
    assert np.abs(K32 - K64).max() <= 1e-5 * np.abs(K64).max()
