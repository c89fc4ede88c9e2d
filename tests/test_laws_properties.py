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
@settings(max_examples=60, deadline=None, suppress_health_check=[HealthCheck.function_scoped_fixture])
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
@settings(max_examples=40, deadline=None, suppress_health_check=[HealthCheck.function_scoped_fixture])
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
