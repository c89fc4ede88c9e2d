"""Learned PCG preconditioner (bartels_lpcg_* in include/bartels_gpu.h).

A 3-layer message-passing network (width 64, BF16 tensor-core GEMMs with FP32
accumulation) over the mesh vertex graph outputs a block-lower-triangular
factor G on the Hessian's pattern; PCG uses M^-1 = G^T G. Its output layers
start at zero, where G is the 3x3 block-Jacobi factor; training (forward,
backward and Adam all in libbartels_gpu.so) lowers the log of Kaporin's
condition number of G H G^T on Hessian / residual pairs that the GPU Newton
solver produces.

The reference has no counterpart: its linear solver is Eigen::SparseLU
(include/search_direction_newton_sparse.h:8).
"""
from __future__ import annotations

import ctypes as C
import math
import os
import time

import numpy as np

from . import _lib
from ._lib import check, lib
from .api import MODELS, Context, MeshPlan, newton_params
from .meshes import kuhn_cube, material_params

H, LAYERS, DX, DE = 64, 3, 4, 10
WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights", "lpcg_neohookean.npz")


def layout():
    """name -> (offset, shape) of the flat FP32 parameter vector (the library's order)."""
    out, o = {}, 0

    def take(name, shape):
        nonlocal o
        out[name] = (o, shape)
        o += int(np.prod(shape))

    take("W0", (DX, H))
    take("b0", (H,))
    for l in range(LAYERS):
        take(f"Wpq{l}", (2 * H, H))
        take(f"We{l}", (DE, H))
        take(f"be{l}", (H,))
        take(f"Wu{l}", (H, 2 * H))
        take(f"bu{l}", (H,))
    take("Wst", (2 * H, H))
    take("Wf", (DE, H))
    take("bf", (H,))
    take("Wo", (H, 9))
    take("bo", (9,))
    take("Wd", (H, 6))
    take("bd", (6,))
    take("Wskip", (DE, 9))
    return out, o


LAYOUT, NPARAMS = layout()


def init_params(seed: int = 0) -> np.ndarray:
    """Random hidden layers, zero output layers (the factor starts at block-Jacobi)."""
    rng = np.random.default_rng(seed)
    theta = np.zeros(NPARAMS, np.float32)

    def put(name, std):
        o, s = LAYOUT[name]
        theta[o:o + int(np.prod(s))] = (std * rng.standard_normal(int(np.prod(s)))).astype(np.float32)

    put("W0", math.sqrt(2.0 / DX))
    for l in range(LAYERS):
        put(f"Wpq{l}", math.sqrt(1.0 / H))
        put(f"We{l}", math.sqrt(1.0 / DE))
        put(f"Wu{l}", math.sqrt(0.5 / (2 * H)))
    put("Wst", math.sqrt(1.0 / H))
    put("Wf", math.sqrt(1.0 / DE))
    return theta


def _ptr(t):
    return C.c_void_p(t.data_ptr())


class LearnedPreconditioner:
    """Network weights and optimiser state on a context (bartels_lpcg)."""

    def __init__(self, ctx: Context | None = None, params: np.ndarray | None = None, seed: int = 0):
        self.ctx = ctx or Context.default()
        if lib().bartels_lpcg_num_params() != NPARAMS:
            raise _lib.BartelsError(_lib.E_INVALID_ARG, "LearnedPreconditioner", "parameter layout mismatch")
        h = C.c_void_p()
        check(lib().bartels_lpcg_create(self.ctx.handle, C.byref(h)), "bartels_lpcg_create")
        self.handle = h
        self.set_params(init_params(seed) if params is None else params)

    def set_params(self, theta):
        th = np.ascontiguousarray(theta, np.float32)
        if th.size != NPARAMS:
            raise ValueError("wrong number of parameters")
        check(lib().bartels_lpcg_set_params(self.handle, th.ctypes.data_as(C.c_void_p)), "bartels_lpcg_set_params")

    def params(self) -> np.ndarray:
        out = np.zeros(NPARAMS, np.float32)
        check(lib().bartels_lpcg_get_params(self.handle, out.ctypes.data_as(C.c_void_p), None),
              "bartels_lpcg_get_params")
        return out

    def grad(self) -> np.ndarray:
        out = np.zeros(NPARAMS, np.float32)
        check(lib().bartels_lpcg_get_params(self.handle, None, out.ctypes.data_as(C.c_void_p)),
              "bartels_lpcg_get_params")
        return out

    def train_step(self, plan: MeshPlan, values, residual=None, nprobes: int = 4, seed: int = 0, lr: float = 1e-3,
                   clip: float = 1.0) -> float:
        """Loss (and gradient; one Adam step when lr > 0) on a plan's Hessian.
        values: FP32 device tensor in the plan's CSR order; residual: FP64 device
        tensor (3nV) or None."""
        loss = C.c_double()
        check(lib().bartels_lpcg_train_step(self.handle, plan.handle, _ptr(values),
                                            None if residual is None else _ptr(residual), nprobes, seed,
                                            C.c_float(lr), C.c_float(clip), C.byref(loss)), "bartels_lpcg_train_step")
        return loss.value

    def outputs(self, plan: MeshPlan, values):
        """(raw (nnzl, 9), G lower storage (9 nnzl,)) for the plan's Hessian values."""
        nl, nu = factor_size(plan)
        raw = np.zeros(9 * nl, np.float32)
        gl = np.zeros(9 * nl, np.float32)
        check(lib().bartels_lpcg_outputs(self.handle, plan.handle, _ptr(values), raw.ctypes.data_as(C.c_void_p),
                                         gl.ctypes.data_as(C.c_void_p)), "bartels_lpcg_outputs")
        return raw.reshape(nl, 9), gl

    def attach(self, plan: MeshPlan, multigrid: bool = False):
        """Make the network the plan's preconditioner: M^-1 = G^T G, or (multigrid)
        the smoother of the finest level of the multigrid V-cycle."""
        kind = _lib.PRECOND_LEARNED_MULTIGRID if multigrid else _lib.PRECOND_LEARNED
        check(lib().bartels_plan_set_preconditioner(plan.handle, kind, self.handle),
              "bartels_plan_set_preconditioner")

    def save(self, path: str, **meta):
        os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
        np.savez(path, params=self.params(), **{k: np.asarray(v) for k, v in meta.items()})

    @classmethod
    def load(cls, path: str = WEIGHTS, ctx: Context | None = None):
        with np.load(path) as z:
            return cls(ctx, params=z["params"])

    def close(self):
        if getattr(self, "handle", None) and getattr(self.ctx, "handle", None):
            lib().bartels_lpcg_destroy(self.handle)
        self.handle = None


def factor_size(plan: MeshPlan):
    nl, nu = C.c_int64(), C.c_int64()
    check(lib().bartels_plan_factor_size(plan.handle, C.byref(nl), C.byref(nu)), "bartels_plan_factor_size")
    return nl.value, nu.value


def use_block_jacobi(plan: MeshPlan):
    check(lib().bartels_plan_set_preconditioner(plan.handle, _lib.PRECOND_BLOCK_JACOBI, None),
          "bartels_plan_set_preconditioner")


def use_multigrid(plan: MeshPlan):
    """Aggregation multigrid V-cycle with block-Jacobi smoothing as the plan's preconditioner."""
    check(lib().bartels_plan_set_preconditioner(plan.handle, _lib.PRECOND_MULTIGRID, None),
          "bartels_plan_set_preconditioner")


def precond_apply(plan: MeshPlan, values, r, z):
    """z = B r with the plan's multigrid preconditioner built for values (device tensors); returns the level count."""
    levels = C.c_int()
    check(lib().bartels_plan_precond_apply_d(plan.ctx.handle, plan.handle, _ptr(values), _ptr(r), _ptr(z),
                                             C.byref(levels)), "bartels_plan_precond_apply_d")
    return levels.value


def mg_info(plan: MeshPlan):
    """Levels of the plan's multigrid hierarchy: {"nodes": [...], "blocks": [...], "coarsest": ...}."""
    n = C.c_int()
    nodes = (C.c_int * 16)()
    blocks = (C.c_int64 * 16)()
    co = C.c_int()
    check(lib().bartels_plan_mg_info(plan.handle, 16, C.byref(n), nodes, blocks, C.byref(co)), "bartels_plan_mg_info")
    return {"nodes": list(nodes[:n.value]), "blocks": list(blocks[:n.value]),
            "coarsest": ["dense", "block-diagonal", "chebyshev"][co.value]}


def plan_pcg(plan: MeshPlan, values, b, x, rel_tol=1e-8, max_iters=20000, inner_rel_tol=0.1, max_refinements=40,
             restart=0):
    """x = H^-1 b on the device with the plan's current preconditioner; returns the report."""
    prm = _lib.PcgParams(rel_tol, max_iters, inner_rel_tol, max_refinements, restart)
    rep = _lib.PcgReport()
    s = lib().bartels_plan_pcg_d(plan.ctx.handle, plan.handle, None if values is None else _ptr(values), _ptr(b),
                                 _ptr(x), C.byref(prm), C.byref(rep))
    if s not in (_lib.OK, _lib.E_NOT_CONVERGED):
        check(s, "bartels_plan_pcg_d")
    return rep


def gemm_bf16(ctx: Context, x, w, bias=None, relu=False, y=None):
    """y = act(x w^T + bias) on the tensor cores; x (M, K) and w (N, K) BF16 device tensors."""
    import torch
    M, K = x.shape
    N = w.shape[0]
    if y is None:
        y = torch.empty(M, N, dtype=torch.float32, device=x.device)
    check(lib().bartels_gemm_bf16_d(ctx.handle, M, N, K, _ptr(x), x.stride(0), _ptr(w),
                                    None if bias is None else _ptr(bias), int(relu), _ptr(y), y.stride(0)),
          "bartels_gemm_bf16_d")
    return y


# ------------------------------------------------------------ training data ---
class System:
    """One (Hessian, residual) pair from a Newton iteration on a plan."""

    def __init__(self, plan, values, residual, meta):
        self.plan, self.values, self.residual, self.meta = plan, values, residual, meta


def sample_configs(count: int, seed: int = 0, n_range=(8, 20), models=("neohookean",), ratio_range=(30.0, 3e4),
                   nu_range=(0.30, 0.48), stretch=0.15, hetero=0.0, hetero_frac=0.5):
    """Implicit-Euler cubes with a spread of stiffness-to-inertia ratios
    E dt^2 / (rho h^2) around the n=96 benchmark's (1.8e3), Poisson ratios,
    initial stretches and (optionally) material models. With hetero > 0 a
    fraction hetero_frac of the cubes gets per-tet stiffness exp(hetero N(0, 1))
    times the cube's E (log-normal heterogeneity)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        n = int(rng.integers(n_range[0], n_range[1] + 1))
        ratio = float(np.exp(rng.uniform(np.log(ratio_range[0]), np.log(ratio_range[1]))))
        young = float(np.exp(rng.uniform(np.log(1e5), np.log(1e7))))
        nu = float(rng.uniform(*nu_range))
        rho, h = 1000.0, 1.0 / n
        dt = math.sqrt(ratio * rho * h * h / young)
        st = rng.uniform(1.0 - stretch, 1.0 + stretch, size=3)
        model = models[int(rng.integers(len(models)))]
        sigma = hetero if (hetero > 0 and rng.uniform() < hetero_frac) else 0.0
        out.append(dict(n=n, young=young, nu=nu, rho=rho, dt=dt, ratio=ratio, stretch=st.tolist(), model=model,
                        hetero=sigma))
    return out


def _cube_params(model, nT, cfg):
    """Per-tet params of a training cube: the cube's (E, nu), times a seeded
    log-normal per-tet factor when cfg["hetero"] > 0 (every law's parameters
    scale with E at fixed nu)."""
    params = material_params(model, nT, cfg["young"], cfg["nu"])
    sigma = cfg.get("hetero", 0.0)
    if sigma > 0:
        f = np.exp(sigma * np.random.default_rng(cfg.get("seed", 0) + 7919).standard_normal(nT))
        if model == "linear_elasticity":
            params[:, 0] *= f
        else:
            params *= f[:, None]
    return params


def newton_systems(ctx: Context, cfg: dict, newton_iters: int = 3, model: str | None = None):
    """Run implicit-Euler Newton on one configuration and return its systems."""
    import torch
    model = model or cfg.get("model", "neohookean")
    dev = torch.device(f"cuda:{ctx.device}")
    V, E = kuhn_cube(cfg["n"])
    plan = MeshPlan(V, E, ctx)
    params = _cube_params(model, len(E), cfg)
    rho = np.full(len(E), cfg["rho"])
    plan.set_element_data(params=params, density=rho)
    vol = None
    pinned = (np.abs(V[:, 2]) <= 1e-12).astype(np.uint8)
    from .api import volume as _volume
    vol = _volume(V, E)
    f_g = plan.const_ext_force(vol, np.array([0.0, 0.0, -9.81 * cfg["rho"]]))
    q_base = (V * np.asarray(cfg["stretch"])[None, :]).ravel()
    plan.set_problem(q_base=q_base, x_hat=np.zeros(3 * len(V)), f_ext=f_g, pinned=pinned)
    dt = cfg["dt"]
    prm = newton_params(model=model, psd_mode=_lib.PSD_SIMPLE_FIX, psd_tol=1e-6, mass_coeff=1.0, scale=dt,
                        force_scale=dt, gradient_tol=1e-8, relative=1, max_iterations=newton_iters)
    stream = ctx.torch_stream()  # torch ops below are ordered with the library's kernels
    with torch.cuda.stream(stream):
        x = torch.zeros(3 * len(V), dtype=torch.float64, device=dev)
        qb = torch.from_numpy(q_base).to(dev)
    nnzb = plan.nnz // 9
    out = []
    g0 = -1.0
    for it in range(newton_iters):
        with torch.cuda.stream(stream):
            values = torch.empty(9 * nnzb, dtype=torch.float32, device=dev)
            q = qb + dt * x
            g = torch.empty_like(x)
        check(lib().bartels_plan_hessian_d(ctx.handle, plan.handle, MODELS[model], _lib.PSD_SIMPLE_FIX, 1e-6, 0,
                                           dt * dt, 1.0, _ptr(q), _ptr(values)), "bartels_plan_hessian_d")
        check(lib().bartels_newton_gradient_d(ctx.handle, plan.handle, C.byref(prm), _ptr(x), _ptr(g)),
              "bartels_newton_gradient_d")
        ctx.synchronize()
        out.append(System(plan, values, g, dict(cfg, newton_iteration=it)))
        done = C.c_int()
        rep = _lib.NewtonReport()
        check(lib().bartels_newton_iterate_d(ctx.handle, plan.handle, C.byref(prm), _ptr(x), C.c_double(g0),
                                             C.byref(done), C.byref(rep)), "bartels_newton_iterate_d")
        g0 = rep.grad_norm0 if rep.grad_norm0 > 0 else g0
        if done.value:
            break
    return out


def packed_newton_systems(ctx: Context, count: int, seed: int, n_range=(8, 40), newton_iters: int = 4,
                          dt: float = 0.01):
    """Yield the (Hessian, residual) pairs of the first newton_iters implicit-Euler
    Newton iterations of `count` instances drawn as bartels_gb300.batched draws
    them (Neo-Hookean cubes, n uniform in n_range, E log-uniform in [1e5, 1e7],
    nu uniform in [0.30, 0.48], per-axis stretch uniform in [0.7, 1.3] plus
    vertex noise, z = 0 pinned, gravity, dt = 0.01), packed into one plan with
    per-instance PCG and line search (bartels_plan_set_segments) and stepped by
    the library's own Newton solver with block-Jacobi PCG. Each yielded System
    holds `count` instance systems; its residual is scaled per instance to unit
    root-mean-square, so that every instance weighs the same in the residual
    probe. The caller closes the plan (System.plan) when it is done with the
    systems."""
    import torch
    from . import batched
    from .api import volume as _volume
    dev = torch.device(f"cuda:{ctx.device}")
    pk = batched.pack(batched.make_instances(count, seed, n_range))
    V, E = pk["V"], pk["E"]
    plan = MeshPlan(V, E, ctx)
    plan.set_element_data(params=pk["params"], density=np.full(len(E), 1000.0))
    f_g = plan.const_ext_force(_volume(V, E), np.array([0.0, 0.0, -9.81 * 1000.0]))
    plan.set_problem(q_base=pk["q_base"].ravel(), x_hat=np.zeros(3 * len(V)), f_ext=f_g, pinned=pk["pinned"])
    voff = np.ascontiguousarray(pk["voff"], np.int32)
    toff = np.ascontiguousarray(pk["toff"], np.int64)
    check(lib().bartels_plan_set_segments(plan.handle, count, voff.ctypes.data_as(C.POINTER(C.c_int)),
                                          toff.ctypes.data_as(C.POINTER(C.c_int64))), "bartels_plan_set_segments")
    prm = newton_params(model="neohookean", psd_mode=_lib.PSD_SIMPLE_FIX, psd_tol=1e-6, mass_coeff=1.0, scale=dt,
                        force_scale=dt, gradient_tol=0.0, relative=0, max_iterations=1 << 30)
    stream = ctx.torch_stream()  # torch ops below are ordered with the library's kernels
    with torch.cuda.stream(stream):
        x = torch.zeros(3 * len(V), dtype=torch.float64, device=dev)
        qb = torch.from_numpy(pk["q_base"].ravel().copy()).to(dev)
        seg = torch.from_numpy(np.repeat(np.arange(count), 3 * np.diff(voff))).to(dev)
        dof = torch.from_numpy(3 * np.diff(voff).astype(np.float64)).to(dev)
    for it in range(newton_iters):
        with torch.cuda.stream(stream):
            values = torch.empty(plan.nnz, dtype=torch.float32, device=dev)
            q = qb + dt * x
            g = torch.empty_like(x)
        check(lib().bartels_plan_hessian_d(ctx.handle, plan.handle, MODELS["neohookean"], _lib.PSD_SIMPLE_FIX,
                                           1e-6, 0, dt * dt, 1.0, _ptr(q), _ptr(values)), "bartels_plan_hessian_d")
        check(lib().bartels_newton_gradient_d(ctx.handle, plan.handle, C.byref(prm), _ptr(x), _ptr(g)),
              "bartels_newton_gradient_d")
        with torch.cuda.stream(stream):
            ss = torch.zeros(count, dtype=torch.float64, device=dev).index_add_(0, seg, g * g)
            g = g * torch.sqrt(dof / torch.clamp(ss, min=1e-300))[seg]
        ctx.synchronize()
        yield System(plan, values, g, dict(instances=count, seed=seed, newton_iteration=it))
        if it + 1 < newton_iters:
            done = C.c_int()
            rep = _lib.NewtonReport()
            check(lib().bartels_newton_iterate_d(ctx.handle, plan.handle, C.byref(prm), _ptr(x), C.c_double(1.0),
                                                 C.byref(done), C.byref(rep)), "bartels_newton_iterate_d")


def train_stream(net: LearnedPreconditioner, ctx: Context, systems: int, steps: int, per_pack: int = 16,
                 n_range=(8, 40), newton_iters: int = 4, pool: int = 8, lr: float = 2e-3, lr_end: float = 1e-4,
                 nprobes: int = 4, seed: int = 0, log=None):
    """Adam on the Kaporin loss over a stream of Newton systems: packs of
    per_pack instances are drawn and stepped (packed_newton_systems) until
    `systems` instance systems have been produced; each packed system enters a
    rolling pool of the `pool` most recent ones, and steps / (packed systems)
    training steps are taken after each arrival on systems drawn from the pool.
    No more than the pool's Hessians (and the plans they belong to) are held."""
    rng = np.random.default_rng(seed)
    packs = max(1, -(-systems // (per_pack * newton_iters)))
    arrivals_total = packs * newton_iters
    hist, recent = [], []
    t0 = time.time()
    produced, done_steps, arrivals, next_log = 0, 0, 0, 0
    def drop_oldest():
        old = recent.pop(0)
        if all(r.plan is not old.plan for r in recent) and old.plan is not current[0]:
            old.plan.close()

    current = [None]
    for k in range(packs):
        for sysm in packed_newton_systems(ctx, per_pack, seed * 100003 + k, n_range, newton_iters):
            current[0] = sysm.plan
            recent.append(sysm)
            if len(recent) > pool:
                drop_oldest()
            produced += per_pack
            arrivals += 1
            # steps owed after this arrival, in integers so that the last
            # arrival reaches exactly `steps`
            target = steps * arrivals // arrivals_total
            while done_steps < target:
                pick = recent[int(rng.integers(len(recent)))]
                a = lr_end + 0.5 * (lr - lr_end) * (1 + math.cos(math.pi * done_steps / max(steps, 1)))
                hist.append(net.train_step(pick.plan, pick.values, pick.residual, nprobes=nprobes,
                                           seed=int(rng.integers(1 << 31)), lr=a, clip=1.0))
                done_steps += 1
            if log and done_steps >= next_log:
                next_log += max(steps // 20, 1)
                log(f"systems {produced:6d}  step {done_steps:6d}  loss {np.mean(hist[-50:]) if hist else 0:.4f}  "
                    f"{time.time() - t0:.1f}s")
        current[0] = None
    while recent:
        drop_oldest()
    return hist, produced


def perturbed_systems(ctx: Context, cfg: dict, count: int = 1, noise: float = 0.02, model: str | None = None):
    """Hessians M + dt^2 K(q) of one configuration at perturbed rest states
    q = X + noise h U(-1, 1) (no residual): the near-rest systems the first
    Newton iterations of a simulation see."""
    import torch
    model = model or cfg.get("model", "neohookean")
    dev = torch.device(f"cuda:{ctx.device}")
    V, E = kuhn_cube(cfg["n"])
    plan = MeshPlan(V, E, ctx)
    plan.set_element_data(params=_cube_params(model, len(E), cfg), density=np.full(len(E), cfg["rho"]))
    plan.set_problem(pinned=(np.abs(V[:, 2]) <= 1e-12).astype(np.uint8))
    rng = np.random.default_rng(cfg.get("seed", 0))
    out = []
    for k in range(count):
        with torch.cuda.stream(ctx.torch_stream()):  # ordered with the library's kernels
            q = torch.from_numpy((V + noise / cfg["n"] * rng.uniform(-1, 1, V.shape)).ravel()).to(dev)
            values = torch.empty(plan.nnz, dtype=torch.float32, device=dev)
        check(lib().bartels_plan_hessian_d(ctx.handle, plan.handle, MODELS[model], _lib.PSD_SIMPLE_FIX, 1e-6, 0,
                                           cfg["dt"] ** 2, 1.0, _ptr(q), _ptr(values)), "bartels_plan_hessian_d")
        out.append(System(plan, values, None, dict(cfg, sample=k)))
    ctx.synchronize()
    return out


def train(net: LearnedPreconditioner, systems, steps: int, lr: float = 2e-3, lr_end: float = 1e-4,
          nprobes: int = 4, seed: int = 0, log=None, residual_probe: bool = True):
    """Adam on the Kaporin loss, cycling through the systems (cosine learning rate)."""
    rng = np.random.default_rng(seed)
    hist = []
    t0 = time.time()
    for s in range(steps):
        sysm = systems[int(rng.integers(len(systems)))]
        a = lr_end + 0.5 * (lr - lr_end) * (1 + math.cos(math.pi * s / max(steps, 1)))
        loss = net.train_step(sysm.plan, sysm.values, sysm.residual if residual_probe else None, nprobes=nprobes,
                              seed=int(rng.integers(1 << 31)), lr=a, clip=1.0)
        hist.append(loss)
        if log and (s % max(steps // 20, 1) == 0 or s == steps - 1):
            log(f"step {s:6d}  loss {np.mean(hist[-50:]):.4f}  lr {a:.2e}  {time.time() - t0:.1f}s")
    return hist
