"""Aggregation multigrid preconditioner on the GPU, through the C ABI.

The V-cycle must be a symmetric positive definite operator; PCG with it must
reach the solution of the same FP32 Hessian system that a direct FP64 solve
gives, in a small fraction of block-Jacobi's iterations, on Kuhn cubes, on a
carved heterogeneous mesh, on packed uneven meshes (a block-diagonal system)
and with the learned factor as the smoother of the finest level. The
reference has no counterpart (its search direction factors the Hessian with
Eigen::SparseLU, src/search_direction_newton_sparse.cpp:12-18), so the
direct solve of the same system is the oracle here."""
import ctypes as C

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as sla

pytestmark = pytest.mark.gpu

SOL_TOL = 1e-6  # PCG to 1e-8 relative residual against the FP64 direct solve of the same FP32 system


def _torch():
    return pytest.importorskip("torch")


def _plan(V, E, params, pinned, density=1000.0):
    import bartels_gb300 as bg
    plan = bg.MeshPlan(V, E)
    plan.set_element_data(params=params, density=np.full(len(E), density))
    plan.set_problem(pinned=pinned.astype(np.uint8))
    return plan


def _hessian(plan, q, coeff=1e-4, psd=True):
    """Implicit-Euler Hessian M + coeff K (coeff = dt^2) at positions q, FP32 on the device."""
    torch = _torch()
    import bartels_gb300 as bg
    from bartels_gb300 import _lib
    qd = torch.from_numpy(np.ascontiguousarray(q).ravel()).cuda()
    vals = torch.empty(plan.nnz, dtype=torch.float32, device="cuda")
    _lib.check(bg.lib().bartels_plan_hessian_d(plan.ctx.handle, plan.handle, _lib.NEOHOOKEAN,
                                               _lib.PSD_SIMPLE_FIX if psd else _lib.PSD_NONE, 1e-6, 0, coeff, 1.0,
                                               C.c_void_p(qd.data_ptr()), C.c_void_p(vals.data_ptr())), "hessian")
    plan.ctx.synchronize()
    return vals


def _cube(n, seed=0, young=2e6, nu=0.45):
    from bartels_gb300.meshes import kuhn_cube, material_params
    V, E = kuhn_cube(n)
    pinned = np.abs(V[:, 2]) < 1e-12
    plan = _plan(V, E, material_params("neohookean", len(E), young, nu), pinned)
    rng = np.random.default_rng(seed)
    q = V + 0.02 / n * rng.uniform(-1, 1, V.shape)
    return plan, V, q, pinned


def _rhs(nV, pinned, seed=1):
    torch = _torch()
    rng = np.random.default_rng(seed)
    b = rng.standard_normal(3 * nV)
    b[np.repeat(pinned, 3)] = 0.0
    return torch.from_numpy(b).cuda()


def _solve(plan, vals, b, kind, net=None, max_iters=20000):
    torch = _torch()
    from bartels_gb300 import lpcg
    if kind == "jacobi":
        lpcg.use_block_jacobi(plan)
    elif kind == "multigrid":
        lpcg.use_multigrid(plan)
    elif kind == "learned_multigrid":
        net.attach(plan, multigrid=True)
    x = torch.zeros_like(b)
    rep = lpcg.plan_pcg(plan, vals, b, x, rel_tol=1e-8, max_iters=max_iters)
    return x.cpu().numpy(), rep


def _direct(plan, vals, b, pinned):
    """FP64 direct solve of the FP32 system restricted to the free DOFs."""
    rp, ci = plan.pattern()
    n = len(rp) - 1
    A = sp.csr_matrix((vals.cpu().numpy().astype(np.float64), ci, rp), shape=(n, n))
    free = np.nonzero(~np.repeat(pinned, 3))[0]
    x = np.zeros(n)
    x[free] = sla.spsolve(A[free][:, free].tocsc(), b.cpu().numpy()[free])
    return x


@pytest.mark.parametrize("n", [6, 12, 20])
def test_multigrid_pcg_matches_direct_solve_in_few_iterations(n):
    plan, V, q, pinned = _cube(n)
    vals = _hessian(plan, q)
    b = _rhs(len(V), pinned)
    x_ref = _direct(plan, vals, b, pinned)
    x_bj, rep_bj = _solve(plan, vals, b, "jacobi")
    x_mg, rep_mg = _solve(plan, vals, b, "multigrid")
    assert rep_bj.converged and rep_mg.converged
    for x in (x_bj, x_mg):
        assert np.linalg.norm(x - x_ref) <= SOL_TOL * np.linalg.norm(x_ref)
        assert np.all(x[np.repeat(pinned, 3)] == 0.0)
    # the V-cycle bounds the iteration count where block-Jacobi's grows with n
    assert rep_mg.iterations <= max(12, 0.3 * rep_bj.iterations), (rep_mg.iterations, rep_bj.iterations)
    plan.close()


def test_vcycle_is_symmetric_positive_definite():
    torch = _torch()
    from bartels_gb300 import lpcg
    plan, V, q, pinned = _cube(10)
    vals = _hessian(plan, q)
    lpcg.use_multigrid(plan)
    mask = torch.from_numpy(np.repeat(~pinned, 3).astype(np.float32)).cuda()
    g = torch.Generator(device="cuda").manual_seed(3)
    rs = [torch.randn(3 * len(V), device="cuda", generator=g) * mask for _ in range(4)]
    zs = []
    for r in rs:
        z = torch.empty_like(r)
        levels = lpcg.precond_apply(plan, vals, r, z)
        assert levels >= 2
        zs.append(z.double())
    info = lpcg.mg_info(plan)
    assert info["nodes"][0] == len(V) and len(info["nodes"]) == levels
    rd = [r.double() for r in rs]
    for i in range(4):
        assert float(rd[i] @ zs[i]) > 0.0
        assert torch.all(zs[i][~mask.bool()] == 0)
        for j in range(i):
            a, c = float(rd[j] @ zs[i]), float(rd[i] @ zs[j])
            scale = float(torch.linalg.norm(rd[i]) * torch.linalg.norm(zs[j]))
            assert abs(a - c) <= 2e-5 * scale, (i, j, a, c)
    # deterministic: the same input gives the same output bit for bit
    z2 = torch.empty_like(rs[0])
    lpcg.precond_apply(plan, vals, rs[0], z2)
    assert torch.equal(z2.double(), zs[0])
    plan.close()


def test_multigrid_follows_a_new_pinned_set():
    plan, V, q, pinned = _cube(10)
    vals = _hessian(plan, q)
    b = _rhs(len(V), pinned)
    x1, rep1 = _solve(plan, vals, b, "multigrid")
    assert rep1.converged
    # pin the x = 0 face as well: the hierarchy is rebuilt for the new free set
    pinned2 = pinned | (np.abs(V[:, 0]) < 1e-12)
    plan.set_problem(pinned=pinned2.astype(np.uint8))
    b2 = _rhs(len(V), pinned2, seed=4)
    x_ref = _direct(plan, vals, b2, pinned2)
    x2, rep2 = _solve(plan, vals, b2, "multigrid")
    assert rep2.converged
    assert np.linalg.norm(x2 - x_ref) <= SOL_TOL * np.linalg.norm(x_ref)
    assert np.all(x2[np.repeat(pinned2, 3)] == 0.0)
    plan.close()


def test_multigrid_on_carved_heterogeneous_mesh():
    from bartels_gb300 import stress_case
    prob = stress_case.build(n=14, seed=0)
    V, E = prob["V"], prob["E"]
    pinned = prob["bottom"] | prob["top"]
    plan = _plan(V, E, prob["params"], pinned)
    rng = np.random.default_rng(2)
    q = V.copy()
    q[:, 2] *= 0.9
    q += 0.002 * rng.uniform(-1, 1, V.shape)
    q[pinned] = V[pinned] * np.array([1, 1, 0.9])
    vals = _hessian(plan, q, coeff=1.0)  # quasi-static: M + K
    b = _rhs(len(V), pinned)
    x_ref = _direct(plan, vals, b, pinned)
    x_bj, rep_bj = _solve(plan, vals, b, "jacobi", max_iters=60000)
    x_mg, rep_mg = _solve(plan, vals, b, "multigrid")
    assert rep_bj.converged and rep_mg.converged
    assert np.linalg.norm(x_mg - x_ref) <= SOL_TOL * np.linalg.norm(x_ref)
    assert rep_mg.iterations <= 0.3 * rep_bj.iterations, (rep_mg.iterations, rep_bj.iterations)
    plan.close()


def test_multigrid_on_packed_uneven_meshes():
    from bartels_gb300 import batched
    inst = batched.make_instances(6, seed=3, n_range=(3, 9))
    pk = batched.pack(inst)
    V, E = pk["V"], pk["E"]
    pinned = pk["pinned"].astype(bool)
    plan = _plan(V, E, pk["params"], pinned)
    vals = _hessian(plan, pk["q_base"].reshape(-1, 3))
    b = _rhs(len(V), pinned)
    x_ref = _direct(plan, vals, b, pinned)
    x_bj, rep_bj = _solve(plan, vals, b, "jacobi")
    x_mg, rep_mg = _solve(plan, vals, b, "multigrid")
    assert rep_bj.converged and rep_mg.converged
    assert np.linalg.norm(x_mg - x_ref) <= SOL_TOL * np.linalg.norm(x_ref)
    assert rep_mg.iterations < rep_bj.iterations
    plan.close()


def test_learned_factor_as_multigrid_smoother():
    """The shipped network's factor as the finest smoother on an unseen cube:
    the V-cycle stays a valid preconditioner (same solution) and needs a small
    fraction of block-Jacobi's iterations."""
    from bartels_gb300 import lpcg
    plan, V, q, pinned = _cube(16, seed=5)
    vals = _hessian(plan, q)
    b = _rhs(len(V), pinned)
    x_ref = _direct(plan, vals, b, pinned)
    net = lpcg.LearnedPreconditioner.load(ctx=plan.ctx)
    x_bj, rep_bj = _solve(plan, vals, b, "jacobi")
    x_mg, rep_mg = _solve(plan, vals, b, "multigrid")
    x_lm, rep_lm = _solve(plan, vals, b, "learned_multigrid", net=net)
    assert rep_lm.converged
    assert np.linalg.norm(x_lm - x_ref) <= SOL_TOL * np.linalg.norm(x_ref)
    assert rep_lm.iterations <= 0.3 * rep_bj.iterations, (rep_lm.iterations, rep_bj.iterations)
    print(f"PCG iterations n=16: block-Jacobi {rep_bj.iterations}, multigrid {rep_mg.iterations}, "
          f"multigrid with the learned smoother {rep_lm.iterations}")
    net.close()
    plan.close()
