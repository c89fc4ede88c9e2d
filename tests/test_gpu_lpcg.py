"""Learned preconditioner on the GPU, through the C ABI: the tcgen05 GEMM, the
network forward and its gradient against the NumPy restatement
(oracle/lpcg.py), the factor-preconditioned PCG, and the gain of a trained
network over block-Jacobi."""
import ctypes as C

import numpy as np
import pytest

from oracle import lpcg as L

pytestmark = pytest.mark.gpu


def _torch():
    return pytest.importorskip("torch")


@pytest.mark.parametrize("N,K", [(128, 64), (64, 128), (64, 64), (128, 128)])
@pytest.mark.parametrize("M", [1, 127, 128, 300, 2053])
def test_tcgen05_gemm_matches_numpy(N, K, M):
    torch = _torch()
    import bartels_gb300 as bg
    from bartels_gb300 import lpcg
    ctx = bg.Context.default()
    g = torch.Generator().manual_seed(M * 1000 + N + K)
    x = torch.randn(M, K, generator=g).to(torch.bfloat16).cuda()
    w = torch.randn(N, K, generator=g).to(torch.bfloat16).cuda()
    b = torch.randn(N, generator=g).cuda()
    for relu in (False, True):
        y = lpcg.gemm_bf16(ctx, x, w, b, relu=relu)
        ref = x.double().cpu().numpy() @ w.double().cpu().numpy().T + b.double().cpu().numpy()
        if relu:
            ref = np.maximum(ref, 0.0)
        err = np.abs(y.cpu().numpy() - ref).max()
        assert err <= 1e-4 * max(1.0, np.abs(ref).max()), (M, N, K, relu, err)


def test_tcgen05_gemm_strided_input():
    torch = _torch()
    import bartels_gb300 as bg
    from bartels_gb300 import lpcg
    ctx = bg.Context.default()
    g = torch.Generator().manual_seed(5)
    big = torch.randn(500, 128, generator=g).to(torch.bfloat16).cuda()
    x = big[:, :64]  # row stride 128, as the library reads bf16(h) out of [h | a]
    w = torch.randn(128, 64, generator=g).to(torch.bfloat16).cuda()
    y = lpcg.gemm_bf16(ctx, x, w)
    ref = x.double().cpu().numpy() @ w.double().cpu().numpy().T
    assert np.abs(y.cpu().numpy() - ref).max() <= 1e-4 * np.abs(ref).max()


def test_tcgen05_gemm_wait_timeout_is_reported_and_the_context_stays_usable():
    """The GEMM's bounded mbarrier wait running out: the probe issues no copy
    and no MMA, so nothing is in flight while its first wait polls a barrier
    that nothing arrives on. The C ABI must report BARTELS_E_TIMEOUT, and a
    normal GEMM right after must still be exact."""
    torch = _torch()
    import bartels_gb300 as bg
    from bartels_gb300 import _lib, lpcg
    ctx = bg.Context.default()
    g = torch.Generator().manual_seed(9)
    x = torch.randn(300, 64, generator=g).to(torch.bfloat16).cuda()
    w = torch.randn(128, 64, generator=g).to(torch.bfloat16).cuda()
    y = torch.full((300, 128), 7.0, device="cuda")
    s = bg.lib().bartels_gemm_bf16_wait_probe_d(ctx.handle, 300, 128, 64, C.c_void_p(x.data_ptr()), 64,
                                                C.c_void_p(w.data_ptr()), C.c_void_p(y.data_ptr()), 128, 16)
    assert s == _lib.E_TIMEOUT
    assert b"bounded wait" in bg.lib().bartels_last_error()
    assert torch.all(y == 7.0)  # the time-out path writes no output
    # the context is unharmed: an ordinary GEMM afterwards
    y2 = lpcg.gemm_bf16(ctx, x, w)
    ref = x.double().cpu().numpy() @ w.double().cpu().numpy().T
    assert np.abs(y2.cpu().numpy() - ref).max() <= 1e-4 * np.abs(ref).max()


def _system(n=4, coeff=1e-2, seed=0):
    """A plan with an implicit-Euler-like Hessian M + coeff K on the device, and
    the same system as oracle blocks."""
    torch = _torch()
    import bartels_gb300 as bg
    from bartels_gb300.meshes import kuhn_cube, material_params
    V, E = kuhn_cube(n)
    rng = np.random.default_rng(seed)
    plan = bg.MeshPlan(V, E)
    params = material_params("neohookean", len(E), 2e6, 0.45)
    plan.set_element_data(params=params, density=np.full(len(E), 1000.0))
    pinned = (np.abs(V[:, 2]) < 1e-12).astype(np.uint8)
    plan.set_problem(pinned=pinned)
    q = (V + 0.02 / n * rng.uniform(-1, 1, V.shape)).ravel()
    qd = torch.from_numpy(q).cuda()
    vals = torch.empty(plan.nnz, dtype=torch.float32, device="cuda")
    from bartels_gb300 import _lib
    _lib.check(bg.lib().bartels_plan_hessian_d(plan.ctx.handle, plan.handle, 0, _lib.PSD_SIMPLE_FIX, 1e-6, 0, coeff,
                                               1.0, C.c_void_p(qd.data_ptr()), C.c_void_p(vals.data_ptr())),
               "hessian")
    plan.ctx.synchronize()
    rp, ci = plan.pattern()
    brp = [0]
    bcol = []
    for v in range(len(V)):
        cols = ci[rp[3 * v]:rp[3 * v + 1]][::3] // 3
        bcol += list(cols)
        brp.append(len(bcol))
    brp, bcol = np.array(brp), np.array(bcol)
    A = L.blocks_from_csr(brp, bcol, vals.cpu().numpy().astype(np.float64))
    g = L.Graph(brp, bcol, pinned.astype(bool))
    return plan, vals, g, A


def _theta(seed=1, head=0.05):
    from bartels_gb300.lpcg import init_params
    th = init_params(seed).astype(np.float64)
    rng = np.random.default_rng(seed + 100)
    for k in ("Wo", "bo", "Wd", "bd"):
        o, s = L.LAYOUT[k]
        th[o:o + int(np.prod(s))] = head * rng.standard_normal(int(np.prod(s)))
    return th.astype(np.float32)


def _lower_index(g):
    """(row v, block b) of each lower block in the library's lower numbering."""
    out = []
    for v in range(g.nV):
        for b in range(g.diag[v] + 1):
            out.append(g.brp[v] + b)
    return np.array(out)


def test_forward_matches_oracle():
    plan, vals, g, A = _system(4)
    from bartels_gb300.lpcg import LearnedPreconditioner
    th = _theta(1)
    net = LearnedPreconditioner(plan.ctx, params=th)
    raw, gl = net.outputs(plan, vals)
    c = L.forward(g, A, th.astype(np.float64), bf=True)
    pos = _lower_index(g)
    ref = np.zeros((len(pos), 9))
    lo = g.lower[pos]
    ref[lo] = c["Gh"][pos[lo]]
    isd = pos == g.dpos[g.row[pos]]
    free_d = isd & ~g.pinned[g.row[pos]]
    ref[free_d, :6] = c["d"][g.row[pos[free_d]]]
    err = np.linalg.norm(raw - ref) / np.linalg.norm(ref)
    assert err < 5e-3, err
    # the factor G = Ghat Linv in lower storage
    Gb = L.factor_blocks(g, c)
    Gb[g.pinned[g.row] | g.pinned[g.bcol]] = 0.0
    mine = np.zeros_like(Gb)
    k = 0
    for v in range(g.nV):
        nl = g.diag[v] + 1
        seg = gl[9 * k:9 * (k + nl)].reshape(3, nl, 3)
        mine[g.brp[v]:g.brp[v] + nl] = seg.transpose(1, 0, 2)
        k += nl
    sel = pos
    e2 = np.linalg.norm(mine[sel] - Gb[sel]) / np.linalg.norm(Gb[sel])
    assert e2 < 5e-3, e2
    net.close()


def test_loss_and_gradient_match_oracle():
    plan, vals, g, A = _system(4)
    from bartels_gb300.lpcg import LearnedPreconditioner
    th = _theta(2)
    net = LearnedPreconditioner(plan.ctx, params=th)
    seed, npr = 12345, 4
    loss = net.train_step(plan, vals, None, nprobes=npr, seed=seed, lr=0.0)
    grad = net.grad().astype(np.float64)
    probes = L.rademacher(seed, npr, 3 * g.nV)
    ref_loss, ref_grad, _ = L.loss_and_grad(g, A, th.astype(np.float64), probes, bf=True)
    assert abs(loss - ref_loss) <= 1e-4 * max(1.0, abs(ref_loss)), (loss, ref_loss)
    cos = grad @ ref_grad / (np.linalg.norm(grad) * np.linalg.norm(ref_grad))
    rel = np.linalg.norm(grad - ref_grad) / np.linalg.norm(ref_grad)
    assert cos > 0.999 and rel < 3e-2, (cos, rel)
    # every parameter group individually
    for name, (o, s) in L.LAYOUT.items():
        n = int(np.prod(s))
        a, b = grad[o:o + n], ref_grad[o:o + n]
        if np.linalg.norm(b) > 1e-6 * np.linalg.norm(ref_grad):
            assert np.linalg.norm(a - b) <= 5e-2 * np.linalg.norm(b), name
    net.close()


def test_zero_head_factor_pcg_equals_block_jacobi():
    torch = _torch()
    plan, vals, g, A = _system(8, coeff=1e-2)
    from bartels_gb300 import lpcg
    net = lpcg.LearnedPreconditioner(plan.ctx)  # output layers zero: G^T G = D^-1 (block-Jacobi)
    b = torch.from_numpy(np.random.default_rng(3).standard_normal(3 * g.nV)).cuda()
    b[torch.from_numpy(np.repeat(g.pinned, 3)).cuda()] = 0.0
    x = torch.zeros_like(b)
    lpcg.use_block_jacobi(plan)
    r_j = lpcg.plan_pcg(plan, vals, b, x)
    net.attach(plan)
    x2 = torch.zeros_like(b)
    r_l = lpcg.plan_pcg(plan, vals, b, x2)
    assert r_j.converged and r_l.converged
    # the factor is stored in BF16, so G^T G is D^-1 to about 3 significant digits
    assert abs(r_j.iterations - r_l.iterations) <= 0.05 * r_j.iterations, (r_j.iterations, r_l.iterations)
    assert r_l.rel_residual <= 1e-8
    assert torch.linalg.norm(x - x2) <= 1e-6 * torch.linalg.norm(x)
    lpcg.use_block_jacobi(plan)
    net.close()


def test_refinement_residual_matches_fp64():
    """The float-float refinement residual (k_resid_blk_ff) against an FP64 host
    residual of the same FP32 matrix, with reliable updates and with restarts."""
    torch = _torch()
    plan, vals, g, A = _system(12, coeff=1e-2)
    from bartels_gb300 import lpcg
    lpcg.use_block_jacobi(plan)
    pin = np.repeat(g.pinned, 3)
    bh = np.random.default_rng(5).standard_normal(3 * g.nV)
    bh[pin] = 0.0
    H = plan.csr(vals.cpu().numpy().astype(np.float64))
    for restart, inner in ((0, 0.1), (1, 1e-4)):
        b = torch.from_numpy(bh).cuda()
        x = torch.zeros_like(b)
        rep = lpcg.plan_pcg(plan, vals, b, x, restart=restart, inner_rel_tol=inner)
        xh = x.cpu().numpy()
        r = bh - H @ xh
        r[pin] = 0.0
        rel = np.linalg.norm(r) / np.linalg.norm(bh)
        assert rep.converged and rel <= 1.001e-8, (restart, rel, rep.rel_residual)
        assert abs(rel - rep.rel_residual) <= 1e-3 * rel + 1e-15, (restart, rel, rep.rel_residual)


def test_residual_probe_training_step_runs():
    torch = _torch()
    plan, vals, g, A = _system(4)
    from bartels_gb300.lpcg import LearnedPreconditioner
    net = LearnedPreconditioner(plan.ctx, params=_theta(3))
    r = torch.from_numpy(np.random.default_rng(1).standard_normal(3 * g.nV)).cuda()
    l0 = net.train_step(plan, vals, r, nprobes=2, seed=1, lr=1e-3)
    assert np.isfinite(l0)
    assert np.all(np.isfinite(net.params()))
    net.close()


def test_training_reduces_pcg_iterations():
    """600 Adam steps (about 1.5 s) on Hessians of small cubes (n = 5..12,
    Neo-Hookean / StVK / corotational, random stiffness and time step, perturbed
    rest states): on an unseen, larger Neo-Hookean cube the learned factor needs
    far fewer PCG iterations than block-Jacobi, and both reach the same solution."""
    torch = _torch()
    import bartels_gb300 as bg
    from bartels_gb300 import lpcg
    ctx = bg.Context.default()
    cfgs = lpcg.sample_configs(12, seed=4, n_range=(5, 12), models=("neohookean", "stvk", "corotational"))
    systems = []
    for k, cfg in enumerate(cfgs):
        cfg["seed"] = k
        systems += lpcg.perturbed_systems(ctx, cfg, count=2)
    net = lpcg.LearnedPreconditioner(ctx, seed=0)
    hist = lpcg.train(net, systems, steps=600, lr=3e-3, lr_end=3e-4, nprobes=8, seed=0)
    assert np.mean(hist[-50:]) < np.mean(hist[:10]) - 0.05
    n = 24
    test_cfg = dict(n=n, young=2e6, nu=0.45, rho=1000.0, dt=0.01 * 96 / n, stretch=[1.0, 1.0, 1.0])
    sysm = lpcg.newton_systems(ctx, test_cfg, newton_iters=1, model="neohookean")[0]
    b = sysm.residual.clone()
    x = torch.zeros_like(b)
    lpcg.use_block_jacobi(sysm.plan)
    rj = lpcg.plan_pcg(sysm.plan, sysm.values, b, x)
    net.attach(sysm.plan)
    x2 = torch.zeros_like(b)
    rl = lpcg.plan_pcg(sysm.plan, sysm.values, b, x2)
    lpcg.use_block_jacobi(sysm.plan)
    assert rj.converged and rl.converged
    assert rl.iterations <= 0.8 * rj.iterations, (rl.iterations, rj.iterations)
    assert torch.linalg.norm(x - x2) <= 1e-6 * torch.linalg.norm(x)
    net.close()


def test_committed_weights_beat_block_jacobi():
    """The shipped weights (bartels_gb300/weights) on a Neo-Hookean cube the
    training never saw (n = 40, the benchmark's E dt^2 / (rho h^2))."""
    torch = _torch()
    import bartels_gb300 as bg
    from bartels_gb300 import lpcg
    ctx = bg.Context.default()
    net = lpcg.LearnedPreconditioner.load(lpcg.WEIGHTS, ctx)
    n = 40
    cfg = dict(n=n, young=2e6, nu=0.45, rho=1000.0, dt=0.01 * 96 / n, stretch=[1.0, 1.0, 1.0])
    for sysm in lpcg.newton_systems(ctx, cfg, newton_iters=2, model="neohookean"):
        b = sysm.residual.clone()
        x = torch.zeros_like(b)
        lpcg.use_block_jacobi(sysm.plan)
        rj = lpcg.plan_pcg(sysm.plan, sysm.values, b, x)
        net.attach(sysm.plan)
        x2 = torch.zeros_like(b)
        rl = lpcg.plan_pcg(sysm.plan, sysm.values, b, x2)
        lpcg.use_block_jacobi(sysm.plan)
        assert rj.converged and rl.converged
        assert rl.iterations <= 0.7 * rj.iterations, (rl.iterations, rj.iterations)
    net.close()


def test_streamed_newton_systems_train_and_release_their_plans():
    """Streaming training on packed Newton systems: 2 packs of 3 instances
    (n = 4..6), 3 Newton iterations each (18 instance systems) through a pool of
    2 packed systems; the loss stays finite, each yielded residual has unit
    root-mean-square per instance, and every pack's plan is closed at the end."""
    torch = _torch()
    import bartels_gb300 as bg
    from bartels_gb300 import lpcg
    ctx = bg.Context.default()
    seen = []
    gen = lpcg.packed_newton_systems(ctx, 3, seed=11, n_range=(4, 6), newton_iters=2)
    for sysm in gen:
        seen.append(sysm)
        assert torch.isfinite(sysm.residual).all()
    plan = seen[0].plan
    r = seen[0].residual.cpu().numpy()
    assert abs(np.sqrt(np.mean(r ** 2)) - 1.0) < 1e-9
    plan.close()
    net = lpcg.LearnedPreconditioner(ctx, seed=0)
    plans = []
    orig = lpcg.packed_newton_systems

    def spy(*a, **k):
        for s in orig(*a, **k):
            plans.append(s.plan)
            yield s
    lpcg.packed_newton_systems = spy
    try:
        hist, produced = lpcg.train_stream(net, ctx, systems=18, steps=6, per_pack=3, n_range=(4, 6),
                                           newton_iters=3, pool=2, nprobes=2, seed=0)
    finally:
        lpcg.packed_newton_systems = orig
    assert produced == 18 and len(hist) == 6 and np.all(np.isfinite(hist))
    assert len({id(p) for p in plans}) == 2 and all(p.handle is None for p in plans)
    net.close()
