"""Batched Newton over many meshes of uneven size packed into one plan.

    python -m bartels_gb300.batched [--count 256] [--nmin 8] [--nmax 40]
                                    [--precond jacobi|multigrid|learned_multigrid|learned]

All instances become one block-diagonal system on a single plan, so every
Newton stage (gradient, fused Hessian, each PCG kernel, line search) is one
launch over all instances, and the PCG inner loop runs as one CUDA graph. The
plan is told where the instances lie (bartels_plan_set_segments), so each
instance keeps its own PCG scalars and its own line-search step: every
instance follows the Newton iterates it would follow alone. Each instance is
checked against its own relative gradient criterion (bartels_segment_sumsq_d
over its vertex range) and stops taking steps once it meets it
(bartels_plan_set_segment_active); the loop ends when every instance has. The
SpMV / factor-pass lane counts come from the autotuner (bartels_plan_autotune),
cached per size bucket.

Instances (seeded): Neo-Hookean Kuhn cubes, n uniform in [nmin, nmax], Young's
modulus log-uniform in [1e5, 1e7] Pa, Poisson ratio uniform in [0.30, 0.48],
initial per-axis stretch uniform in [0.7, 1.3] plus vertex noise 0.01 x edge,
rho = 1000, z = 0 face pinned, gravity, one implicit-Euler step (dt = 0.01)
from rest velocity. FP32 Hessians / PCG with FP64 residuals.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import time

import numpy as np


def make_instances(count=256, seed=0, n_range=(8, 40)):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        n = int(rng.integers(n_range[0], n_range[1] + 1))
        out.append(dict(n=n, young=float(np.exp(rng.uniform(np.log(1e5), np.log(1e7)))),
                        nu=float(rng.uniform(0.30, 0.48)), stretch=rng.uniform(0.7, 1.3, 3),
                        noise_seed=int(rng.integers(1 << 31))))
    return out


def pack(instances):
    """Concatenate the instances: V, E, per-tet params / density, pinned, q_base,
    vertex offsets (count + 1) and tet offsets."""
    from .meshes import kuhn_cube, material_params
    Vs, Es, Ps, pins, qs, voff, toff = [], [], [], [], [], [0], [0]
    for inst in instances:
        V, E = kuhn_cube(inst["n"])
        h = 1.0 / inst["n"]
        rng = np.random.default_rng(inst["noise_seed"])
        q = V * inst["stretch"][None, :] + 0.01 * h * rng.uniform(-1, 1, V.shape)
        q[:, 2] = np.where(V[:, 2] <= 1e-12, 0.0, q[:, 2])  # pinned face stays on z = 0
        Vs.append(V)
        Es.append(E + voff[-1])
        Ps.append(material_params("neohookean", len(E), inst["young"], inst["nu"]))
        pins.append((V[:, 2] <= 1e-12).astype(np.uint8))
        qs.append(q)
        voff.append(voff[-1] + len(V))
        toff.append(toff[-1] + len(E))
    return dict(V=np.concatenate(Vs), E=np.concatenate(Es).astype(np.int32), params=np.concatenate(Ps),
                pinned=np.concatenate(pins), q_base=np.concatenate(qs), voff=np.array(voff, np.int32),
                toff=np.array(toff, np.int64))


def solve(packed, dt=0.01, tol=1e-8, max_newton=60, precond="jacobi", net=None, autotune=True, log=None):
    """One implicit-Euler step of every instance; returns (stats, per-instance
    relative gradient norms, x on the host)."""
    import torch
    import bartels_gb300 as bg
    from bartels_gb300 import _lib
    L = bg.lib()
    ctx = bg.Context.default()
    V, E = packed["V"], packed["E"]
    nV, nT, ns = len(V), len(E), len(packed["voff"]) - 1
    t0 = time.perf_counter()
    plan = bg.MeshPlan(V, E, ctx)
    rho = 1000.0
    plan.set_element_data(params=packed["params"], density=np.full(nT, rho))
    from .api import volume as _volume
    f_g = plan.const_ext_force(_volume(V, E), np.array([0.0, 0.0, -9.81 * rho]))
    plan.set_problem(q_base=packed["q_base"].ravel(), x_hat=np.zeros(3 * nV), f_ext=f_g, pinned=packed["pinned"])
    voff_h = np.ascontiguousarray(packed["voff"], np.int32)
    toff_h = np.ascontiguousarray(packed["toff"], np.int64)
    _lib.check(L.bartels_plan_set_segments(plan.handle, ns, voff_h.ctypes.data_as(C.POINTER(C.c_int)),
                                           toff_h.ctypes.data_as(C.POINTER(C.c_int64))), "set_segments")
    t_setup = time.perf_counter() - t0
    prm = bg.newton_params(model="neohookean", psd_mode=_lib.PSD_SIMPLE_FIX, psd_tol=1e-6, mass_coeff=1.0, scale=dt,
                           force_scale=dt, gradient_tol=0.0, relative=0, max_iterations=1 << 30)
    dev = torch.device(f"cuda:{ctx.device}")
    with torch.cuda.stream(ctx.torch_stream()):  # ordered with the library's kernels
        x = torch.zeros(3 * nV, dtype=torch.float64, device=dev)
        g = torch.empty_like(x)
        off = torch.from_numpy(packed["voff"]).to(dev)
        ss = torch.empty(ns, dtype=torch.float64, device=dev)
    xp, gp = C.c_void_p(x.data_ptr()), C.c_void_p(g.data_ptr())

    def inst_norms():
        _lib.check(L.bartels_newton_gradient_d(ctx.handle, plan.handle, C.byref(prm), xp, gp), "gradient")
        _lib.check(L.bartels_segment_sumsq_d(ctx.handle, ns, C.c_void_p(off.data_ptr()), gp,
                                             C.c_void_p(ss.data_ptr())), "segment_sumsq")
        ctx.synchronize()
        return np.sqrt(ss.cpu().numpy())

    tuned = None
    if autotune:
        with torch.cuda.stream(ctx.torch_stream()):
            q = torch.from_numpy(packed["q_base"].ravel()).to(dev)
        hc, hb = C.c_int(), C.c_int()
        _lib.check(L.bartels_plan_autotune_hessian(ctx.handle, plan.handle, 0, C.c_void_p(q.data_ptr()), 0,
                                                   C.byref(hc), C.byref(hb)), "autotune_hessian")
        _lib.check(L.bartels_plan_hessian_d(ctx.handle, plan.handle, 0, _lib.PSD_SIMPLE_FIX, 1e-6, 0, dt * dt, 1.0,
                                            C.c_void_p(q.data_ptr()), None), "hessian")
        a, b = C.c_int(), C.c_int()
        t1 = time.perf_counter()
        _lib.check(L.bartels_plan_autotune(ctx.handle, plan.handle, None, 0, C.byref(a), C.byref(b)), "autotune")
        tuned = dict(spmv_lanes=a.value, factor_lanes=b.value, hessian_chunk_vertices=hc.value, psd_block=hb.value,
                     seconds=round(time.perf_counter() - t1, 3))
    if precond == "learned":
        net.attach(plan)
    elif precond == "learned_multigrid":
        net.attach(plan, multigrid=True)
    elif precond == "multigrid":
        _lib.check(L.bartels_plan_set_preconditioner(plan.handle, _lib.PRECOND_MULTIGRID, None), "precond")
    if precond in ("multigrid", "learned_multigrid"):
        prm.pcg.inner_rel_tol = 1e-2
    g0 = inst_norms()
    rep = _lib.NewtonReport()
    its = 0
    rel = np.ones(ns)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    while its < max_newton:
        done = C.c_int()
        _lib.check(L.bartels_newton_iterate_d(ctx.handle, plan.handle, C.byref(prm), xp, C.c_double(1.0),
                                              C.byref(done), C.byref(rep)), "newton_iterate")
        its += 1
        rel = inst_norms() / np.maximum(g0, 1e-300)
        active = (rel > tol).astype(np.uint8)
        _lib.check(L.bartels_plan_set_segment_active(plan.handle, active.ctypes.data_as(C.c_void_p)), "active")
        if log:
            log(json.dumps(dict(newton=its, max_rel=float(rel.max()), median_rel=float(np.median(rel)),
                                active=int(active.sum()), pcg=rep.last_pcg_iterations, alpha=rep.last_alpha)))
        if not active.any():
            break
    torch.cuda.synchronize()
    t_solve = time.perf_counter() - t1
    stats = dict(instances=ns, vertices=nV, tets=nT, newton=its, pcg=rep.pcg_iterations,
                 converged=int((rel <= tol).sum()), max_rel_grad=float(rel.max()), seconds=t_solve,
                 newton_per_s=its / t_solve, tets_x_newton_per_s=nT * its / t_solve, setup_s=t_setup,
                 autotune=tuned, fallbacks=rep.precond_fallbacks, kernel_launches=ctx.kernel_launches)
    xh = x.cpu().numpy()
    plan.close()
    return stats, rel, xh


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--count", type=int, default=256)
    ap.add_argument("--nmin", type=int, default=8)
    ap.add_argument("--nmax", type=int, default=40)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--precond", default="jacobi", choices=["jacobi", "multigrid", "learned_multigrid", "learned"])
    ap.add_argument("--tol", type=float, default=1e-8)
    args = ap.parse_args(argv)
    t = time.time()
    inst = make_instances(args.count, args.seed, (args.nmin, args.nmax))
    packed = pack(inst)
    print(json.dumps(dict(instances=args.count, vertices=len(packed["V"]), tets=len(packed["E"]),
                          pack_s=round(time.time() - t, 1))), flush=True)
    net = None
    if args.precond in ("learned", "learned_multigrid"):
        import bartels_gb300 as bg
        from bartels_gb300 import lpcg
        net = lpcg.LearnedPreconditioner.load(lpcg.WEIGHTS, bg.Context.default())
    stats, rel, _ = solve(packed, tol=args.tol, precond=args.precond, net=net,
                          log=lambda s: print(s, flush=True))
    print(json.dumps(stats), flush=True)
    return stats


if __name__ == "__main__":
    main()
