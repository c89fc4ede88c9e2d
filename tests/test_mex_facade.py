"""MATLAB-gateway facade (include/bartels_mex.h) without a GPU: the routine
list covers the reference's gateways on this path, fixed_point_constraint_matrix
(host-only integer work) returns MATLAB's compressed columns of the oracle's P,
and malformed gateway arguments are rejected before any device work."""
import numpy as np
import pytest

from conftest import gpu_available

import bartels_gb300 as bg
from bartels_gb300 import _lib, mex

MODELS = ["neohookean", "stvk", "corotational", "arap"]
# matlab/<name>.cpp gateways of the tet and triangle families and the pointwise
# laws (the muscle model and linear_*_B / _F are outside this library)
GATEWAYS = (
    ["linear_tetmesh_dphi_dX", "linear_tetmesh_mass_matrix", "fixed_point_constraint_matrix",
     "linear_tetmesh_linear_elasticity_dq2", "linear_tri2dmesh_dphi_dX", "linear_tri2dmesh_mass_matrix",
     "linear_tri2dmesh_linear_elasticity_dq2", "linear_tri3dmesh_dphi_dX", "linear_tri3dmesh_stvk_dq2"]
    + [f"linear_tetmesh_{m}_{w}" for m in MODELS for w in ("q", "dq", "dq2")]
    + [f"linear_tri2dmesh_{m}_{w}" for m in MODELS for w in ("q", "dq", "dq2")]
    + ["dpsi_neohookean_dF", "d2psi_neohookean_dF2", "d2psi_stvk_dF2"]
)


def test_routine_list_covers_the_gateways():
    assert sorted(mex.routines()) == sorted(GATEWAYS)


def test_fixed_point_constraint_matrix_in_matlab_layout(oracle):
    rng = np.random.default_rng(3)
    for nV, dim in ((1, 3), (7, 3), (30, 3), (12, 2)):
        fixed = np.sort(rng.choice(nV, size=rng.integers(0, nV), replace=False))
        V = rng.standard_normal((nV, dim))
        P = mex.call("fixed_point_constraint_matrix", V, fixed + 1.0)   # 1-based, as MATLAB passes it
        R = oracle.fixed_point_constraint_matrix(nV, fixed.astype(np.int32), dim=dim).tocsc()
        assert P.shape == R.shape == (dim * (nV - len(fixed)), dim * nV)
        assert np.array_equal(P.indptr, R.indptr) and np.array_equal(P.indices, R.indices)
        assert np.array_equal(P.data, R.data)


def test_fixed_point_rejects_bad_indices():
    V = np.zeros((5, 3))
    for bad in ([0.0], [6.0], [1.5], [3.0, 2.0]):
        with pytest.raises(bg.BartelsError):
            mex.call("fixed_point_constraint_matrix", V, np.array(bad))


def _tet_args():
    V, E = bg.meshes.kuhn_cube(1)
    params = np.tile([1e5, 2e5], (len(E), 1))
    return V, E + 1.0, V.ravel(), np.zeros((len(E), 12)), np.full(len(E), 1 / 6), params


@pytest.mark.parametrize("mutate, msg", [
    (lambda a: a.__setitem__(1, a[1] - 1.0), "E"),            # 0-based E
    (lambda a: a.__setitem__(1, a[1] + 0.5), "E"),            # not integral
    (lambda a: a.__setitem__(0, a[0][:, :2]), "V"),           # V with 2 columns for a tet routine
    (lambda a: a.__setitem__(2, a[2][:-1]), "q"),
    (lambda a: a.__setitem__(3, a[3][:, :9]), "dphidX"),
    (lambda a: a.__setitem__(4, a[4][:-1]), "volumes"),
    (lambda a: a.__setitem__(5, a[5][:, :1]), "params"),      # one column is ARAP only
])
def test_gateway_arguments_are_validated_before_device_work(mutate, msg):
    args = list(_tet_args())
    mutate(args)
    with pytest.raises(bg.BartelsError) as ei:
        mex.call("linear_tetmesh_neohookean_dq2", *args)
    assert ei.value.status == _lib.E_INVALID_ARG and msg in str(ei.value)


def test_unknown_routine_and_missing_arguments():
    with pytest.raises(bg.BartelsError) as ei:
        mex.call("linear_tetmesh_muscle_dq2", np.zeros((4, 3)))
    assert "unknown routine" in str(ei.value)
    with pytest.raises(bg.BartelsError) as ei:
        mex.call("linear_tetmesh_neohookean_q", *_tet_args()[:5])
    assert "takes 6 arguments" in str(ei.value)


def test_valid_call_without_gpu_reports_no_device():
    if gpu_available():
        pytest.skip("a GPU is present")
    with pytest.raises(bg.BartelsError) as ei:
        mex.call("linear_tetmesh_arap_q", *_tet_args()[:5], _tet_args()[5][:, :1])  # ARAP: one column is fine
    assert ei.value.status == _lib.E_NO_DEVICE


def test_pointwise_gateways_validate_shapes():
    E = np.ones((4, 4))
    with pytest.raises(bg.BartelsError) as ei:
        mex.call("d2psi_neohookean_dF2", E, np.zeros((3, 9)), np.ones((4, 2)))
    assert "F" in str(ei.value)
    with pytest.raises(bg.BartelsError) as ei:
        mex.call("dpsi_neohookean_dF", E, np.zeros((4, 9)), np.ones((4, 1)))
    assert "params" in str(ei.value)


def test_facade_layout_with_a_stand_in_abi():
    """mex.cpp linked against a stand-in C ABI with unsymmetric values
    (tests/mex_fake_abi.cpp): compressed columns carry H(i, j), q reaches the
    ABI unshifted, dense and block-diagonal layouts, index checks, the plan
    cache and its eviction."""
    import os
    import subprocess
    from conftest import ROOT
    out_dir = os.path.join(ROOT, "tests", "_build")
    os.makedirs(out_dir, exist_ok=True)
    exe = os.path.join(out_dir, "mex_fake_abi")
    subprocess.check_call(["g++", "-std=c++17", "-O1", os.path.join(ROOT, "tests", "mex_fake_abi.cpp"),
                           os.path.join(ROOT, "bartels_gb300", "csrc", "mex.cpp"), "-I", os.path.join(ROOT, "include"),
                           "-o", exe])
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "mex facade ok" in r.stdout, r.stderr
