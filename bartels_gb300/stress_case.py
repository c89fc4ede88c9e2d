"""Ill-conditioned heterogeneous stress case: learned vs block-Jacobi PCG.

    python -m bartels_gb300.stress_case [--n 64] [--steps 10] [--seed 0]

Mesh: the n^3 Kuhn cube carved to the union of 12 random spheres (radius
U[0.15, 0.35]), largest connected component. Material: Neo-Hookean, per-tet
Young's modulus log-normal (median 1e6 Pa, sigma 1.0 in ln) with stiff
spherical inclusions at 100x, Poisson ratio 0.47. Load: 50% axial compression:
the bottom face (min z) pinned and the top face (max z) prescribed, applied in
load steps (each starts from the previous solution compressed affinely in z),
quasi-static Newton per step to 1e-5 relative gradient norm (projected Newton
converges only linearly here: the PSD projection is active at the compressed
equilibrium, so the tolerance and a 40-iteration cap are set for that). Each Newton system is solved by PCG to 1e-8
relative residual with block-Jacobi, the learned factor, the multigrid V-cycle
and the V-cycle with the learned smoother (block-Jacobi as fallback). Reported: Newton and PCG iteration counts, fallbacks, time, and
the energy of the final state (tests/test_gpu_stress.py checks the final
state against the FP64 CPU restatement). Synthetic, seeded inputs.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import time

import numpy as np


def build(n=64, seed=0):
    from .meshes import carved_cube, lame_from_young
    rng = np.random.default_rng(seed)
    centers = rng.uniform(0.0, 1.0, (12, 3))
    radii = rng.uniform(0.15, 0.35, 12)
    V, E, cent = carved_cube(n, centers, radii)
    young = 1e6 * np.exp(rng.standard_normal(len(E)))
    inc_c = rng.uniform(0.1, 0.9, (8, 3))
    inc_r = rng.uniform(0.04, 0.08, 8)
    inside = (((cent[:, None, :] - inc_c[None, :, :]) ** 2).sum(axis=2) <= inc_r[None, :] ** 2).any(axis=1)
    young[inside] *= 100.0
    lam, mu = lame_from_young(young, 0.47)
    params = np.stack([0.5 * mu, 0.5 * lam], axis=1)  # Neo-Hookean (C, D) per tet
    z = V[:, 2]
    bottom = np.abs(z - z.min()) <= 1e-9
    top = np.abs(z - z.max()) <= 1e-9
    return dict(V=V, E=E, params=params, bottom=bottom, top=top, inclusion_tets=int(inside.sum()),
                young_range=(float(young.min()), float(young.max())))


def run(prob, precond, net=None, steps=10, compression=0.5, gradient_tol=1e-5, max_newton=40, log=print):
    import torch
    import bartels_gb300 as bg
    from bartels_gb300 import _lib
    L = bg.lib()
    ctx = bg.Context.default()
    V, E = prob["V"], prob["E"]
    plan = bg.MeshPlan(V, E, ctx)
    plan.set_element_data(params=prob["params"])
    pinned = (prob["bottom"] | prob["top"]).astype(np.uint8)
    if precond == "learned":
        net.attach(plan)
    elif precond == "learned_multigrid":
        net.attach(plan, multigrid=True)
    elif precond == "multigrid":
        _lib.check(L.bartels_plan_set_preconditioner(plan.handle, _lib.PRECOND_MULTIGRID, None), "precond")
    prm = bg.newton_params(model="neohookean", psd_mode=_lib.PSD_SIMPLE_FIX, psd_tol=1e-6, mass_coeff=0.0, scale=1.0,
                           force_scale=0.0, gradient_tol=gradient_tol, relative=1, max_iterations=max_newton)
    prm.pcg.max_iters = 60000
    if precond in ("multigrid", "learned_multigrid"):
        prm.pcg.inner_rel_tol = 1e-2
    zmin, zmax = V[:, 2].min(), V[:, 2].max()
    q = V.copy()
    x = torch.zeros(3 * len(V), dtype=torch.float64, device="cuda")
    rows = []
    tot = dict(newton=0, pcg=0, fallbacks=0, seconds=0.0, pcg_failures=0)
    c_prev = 0.0
    for s in range(1, steps + 1):
        c = compression * s / steps
        # affine prediction in z about the bottom face; top face at its prescribed height
        q[:, 2] = zmin + (q[:, 2] - zmin) * (1.0 - c) / (1.0 - c_prev)
        c_prev = c
        plan.set_problem(q_base=q.ravel(), pinned=pinned)
        x.zero_()
        rep = _lib.NewtonReport()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s_ = L.bartels_newton_solve_d(ctx.handle, plan.handle, C.byref(prm), C.c_void_p(x.data_ptr()), C.byref(rep))
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        _lib.check(s_, "bartels_newton_solve_d")
        q = q + x.cpu().numpy().reshape(-1, 3)
        row = dict(precond=precond, step=s, compression=c, newton=rep.iterations, pcg=rep.pcg_iterations,
                   fallbacks=rep.precond_fallbacks, pcg_failures=rep.pcg_failures,
                   converged=rep.status == _lib.CONVERGED, rel_grad=rep.grad_norm / max(rep.grad_norm0, 1e-300),
                   seconds=round(dt, 3))
        rows.append(row)
        log(json.dumps(row))
        tot["newton"] += rep.iterations
        tot["pcg"] += rep.pcg_iterations
        tot["fallbacks"] += rep.precond_fallbacks
        tot["pcg_failures"] += rep.pcg_failures
        tot["seconds"] += dt
    # final state (FP64 energy; its check against the FP64 CPU restatement is
    # tests/test_gpu_stress.py)
    tot.update(energy=plan.q("neohookean", q.ravel()), pcg_per_newton=tot["pcg"] / max(tot["newton"], 1))
    plan.close()
    return rows, tot, q


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=64)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--weights", default=None)
    ap.add_argument("--gradient-tol", type=float, default=1e-5)
    ap.add_argument("--preconds", default="jacobi,learned,multigrid,learned_multigrid",
                    help="comma-separated preconditioners to compare")
    args = ap.parse_args(argv)
    import bartels_gb300 as bg
    from bartels_gb300 import lpcg
    t = time.time()
    prob = build(args.n, args.seed)
    print(json.dumps(dict(vertices=len(prob["V"]), tets=len(prob["E"]), inclusion_tets=prob["inclusion_tets"],
                          young_range=prob["young_range"], bottom=int(prob["bottom"].sum()),
                          top=int(prob["top"].sum()), build_s=round(time.time() - t, 1))), flush=True)
    net = lpcg.LearnedPreconditioner.load(args.weights or lpcg.WEIGHTS, bg.Context.default())
    out = {}
    for pc in args.preconds.split(","):
        _, tot, _ = run(prob, pc, net, steps=args.steps, gradient_tol=args.gradient_tol,
                        log=lambda s: print(s, flush=True))
        out[pc] = tot
        print(json.dumps(dict(summary=pc, **tot)), flush=True)
    for pc in out.copy():
        if pc != "jacobi" and "jacobi" in out:
            out[f"{pc}_over_jacobi_seconds"] = out["jacobi"]["seconds"] / out[pc]["seconds"]
    print(json.dumps(out), flush=True)
    return out


if __name__ == "__main__":
    main()
