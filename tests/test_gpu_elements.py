"""Per-element parity against the FP64 oracle, through the C ABI.

Energies: bartels_tetmesh_q_elements_d gives every tet's psi(F) vol (the
reference's linear_tet_*_q, src/linear_tet_neohookean_q.cpp:5-18). Gradients
and Hessians: an "exploded" copy of a mesh, in which every tet has its own
four vertices, makes the assembled gradient and Hessian block diagonal, so
each 12-vector of the gradient and each 12x12 diagonal block of the Hessian is
one element's contribution exactly as the library's fused kernels computed it
(linear_tet_*_dq / _dq2, src/linear_tet_neohookean_dq2.cpp:5-23, with the
simple_psd_fix callback, src/simple_psd_fix.cpp:9-19). Bounds per element:
FP64 energy and gradient 1e-10 relative, FP32 Hessian 1e-5 relative in the
Frobenius norm, every law, with and without the projection, including
strongly compressed StVK and a sample of the 96^3-cell cube's tets."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ELEM_TOL64 = 1e-10  # FP64 element energy / gradient, relative per element
ELEM_TOL32 = 1e-5   # FP32 element Hessian, relative Frobenius per element

MODELS = ["neohookean", "stvk", "corotational", "neohookean_isochoric", "arap", "linear_elasticity"]


def _explode(V, E, q):
    """Every tet with its own four vertices: (V, E, q) of the exploded mesh."""
    Vx = V[E].reshape(-1, 3)
    Ex = np.arange(4 * len(E), dtype=np.int32).reshape(-1, 4)
    qx = q.reshape(-1, 3)[E].reshape(-1, 3)
    return Vx, Ex, qx


def _state(kind, n=3, seed=0):
    from bartels_gb300.meshes import kuhn_cube
    V, E = kuhn_cube(n)
    rng = np.random.default_rng(seed)
    h = 1.0 / n
    if kind == "moderate":
        A = np.eye(3) + 0.15 * rng.standard_normal((3, 3))
        q = V @ A.T + 0.1 * h * rng.uniform(-1, 1, V.shape)
    elif kind == "compressed":  # 60% in z, 20% vertex noise
        q = V * np.array([1.0, 1.0, 0.6]) + 0.2 * h * rng.uniform(-1, 1, V.shape)
    else:
        raise ValueError(kind)
    return V, E, q


def _relerr(a, b, axis):
    """Per-element relative error with a floor at 1e-12 of the largest element."""
    num = np.linalg.norm(a - b, axis=axis)
    den = np.linalg.norm(b, axis=axis)
    return num / np.maximum(den, 1e-12 * den.max())


def _check_elements(oracle, model, V, E, q, psd_tols):
    torch = pytest.importorskip("torch")
    import bartels_gb300 as bg
    from bartels_gb300 import _lib
    from bartels_gb300.meshes import material_params
    params = material_params(model, len(E), 2e6, 0.45)
    Vx, Ex, qx = _explode(V, E, q)
    plan = bg.MeshPlan(Vx, Ex)
    # the plan stores linear elasticity's parameters as the Lame pair (the
    # entry points that take params convert the reference's (E, nu) to it)
    stored = params
    if model == "linear_elasticity":
        young, nu = params[:, 0], params[:, 1]
        stored = np.stack([young * nu / ((1 + nu) * (1 - 2 * nu)), young / (2 * (1 + nu))], axis=1)
    plan.set_element_data(params=stored)
    dphi, vol = oracle.dphi_dX(Vx, Ex), oracle.volume(Vx, Ex)
    # energies
    q_d = torch.from_numpy(qx.ravel().copy()).cuda()
    e_d = torch.empty(len(E), dtype=torch.float64, device="cuda")
    _lib.check(bg.lib().bartels_tetmesh_q_elements_d(plan.ctx.handle, plan.handle, bg.api.MODELS[model],
                                                     C.c_void_p(q_d.data_ptr()), C.c_void_p(e_d.data_ptr())),
               "bartels_tetmesh_q_elements_d")
    plan.ctx.synchronize()
    e_ref = oracle.tetmesh_q_elements(model, Ex, qx.ravel(), dphi, vol, params)
    err_e = _relerr(e_d.cpu().numpy()[:, None], e_ref[:, None], axis=1)
    assert err_e.max() <= ELEM_TOL64, (model, "energy", err_e.max())
    # gradients: one 12-vector per exploded tet
    g = plan.dq(model, qx.ravel()).reshape(len(E), 12)
    g_ref = oracle.tetmesh_dq(model, len(Vx), Ex, qx.ravel(), dphi, vol, params).reshape(len(E), 12)
    err_g = _relerr(g, g_ref, axis=1)
    assert err_g.max() <= ELEM_TOL64, (model, "gradient", err_g.max())
    # Hessians: the 12x12 diagonal blocks
    worst = {}
    for tol in psd_tols:
        H = plan.dq2(model, qx.ravel(), psd_tol=tol).tocsr()
        assert H.nnz == 144 * len(E)  # nothing outside the elements' own blocks
        K = np.stack([H[12 * t:12 * t + 12, 12 * t:12 * t + 12].toarray() for t in range(len(E))])
        K_ref = oracle.tetmesh_dq2_elements(model, Ex, qx.ravel(), dphi, vol, params, psd_tol=tol)
        err_h = _relerr(K.reshape(len(E), -1), K_ref.reshape(len(E), -1), axis=1)
        assert err_h.max() <= ELEM_TOL32, (model, tol, "hessian", err_h.max())
        worst[tol] = float(err_h.max())
    plan.close()
    return worst


@pytest.mark.parametrize("model", MODELS)
def test_per_element_parity_moderate_deformation(oracle, model):
    V, E, q = _state("moderate")
    _check_elements(oracle, model, V, E, q, [None, 1e-6])


@pytest.mark.parametrize("model", ["stvk", "neohookean", "corotational"])
def test_per_element_parity_strong_compression(oracle, model):
    V, E, q = _state("compressed", n=4, seed=3)
    worst = _check_elements(oracle, model, V, E, q, [None, 1e-6, 1e-3])
    print(model, "worst per-element Hessian error", worst)


def test_per_element_parity_on_a_sample_of_the_full_cube(oracle):
    """20,000 tets drawn from the 96^3-cell cube compressed to 60% with 20%
    vertex noise (the full-size StVK state), exploded and checked element by
    element with the projection on."""
    from bartels_gb300.meshes import kuhn_cube
    V, E = kuhn_cube(96)
    rng = np.random.default_rng(11)
    h = 1.0 / 96
    q = V * np.array([1.0, 1.0, 0.6]) + 0.2 * h * rng.uniform(-1, 1, V.shape)
    pick = np.sort(rng.choice(len(E), 20000, replace=False))
    worst = _check_elements(oracle, "stvk", V, E[pick], q, [1e-6])
    print("n=96 sample, worst per-element Hessian error", worst)
