"""Train the learned PCG preconditioner on the GPU and write its weights.

    python -m bartels_gb300.train_lpcg --kind rest --no-residual --models neohookean,stvk,corotational \
        --probes 8 --seed 0 --newton-iters 2 --systems 48 --nmin 12 --nmax 40 --steps 12000 \
        --hetero 1.0 --hetero-frac 0.5 --lr 3e-3 --eval 40,96 --out bartels_gb300/weights/lpcg_neohookean.npz
        (the recipe of the shipped weights)
    python -m bartels_gb300.train_lpcg --systems 0 --steps 0 --init bartels_gb300/weights/lpcg_neohookean.npz --eval 96
        (evaluation only: PCG iterations and seconds, learned vs block-Jacobi)
    python -m bartels_gb300.train_lpcg --kind stream --systems 20000 --per-pack 16 --newton-iters 4 --nmin 8 \
        --nmax 40 --steps 6000 --probes 4 --lr 2e-3 --eval 40,96 --out weights.npz
        (Newton systems of packed batched-style instances, streamed: 20k instance systems, never all held)

Training systems are (Hessian, residual) pairs from implicit-Euler Newton
iterations on Neo-Hookean Kuhn cubes of random size, stiffness, Poisson ratio,
time step and initial stretch (bartels_gb300.lpcg.sample_configs), produced by
the library's own Newton solver. The network, its loss gradient and the Adam
updates run in libbartels_gpu.so. After training, PCG iteration counts with
the learned factor and with block-Jacobi are compared on held-out cubes whose
stiffness-to-inertia ratio E dt^2 / (rho h^2) matches the n=96 benchmark.
"""
from __future__ import annotations

import argparse
import json
import math
import time

import numpy as np


def evaluate(ctx, net, sizes, model="neohookean", newton_iters=2, log=print):
    """PCG iterations (learned vs block-Jacobi) on Neo-Hookean cubes whose
    E dt^2 / (rho h^2) equals the n=96 benchmark's."""
    import torch
    from . import lpcg
    out = []
    for n in sizes:
        cfg = dict(n=n, young=2e6, nu=0.45, rho=1000.0, dt=0.01 * 96 / n, ratio=1843.0, stretch=[1.0, 1.0, 1.0])
        for sysm in lpcg.newton_systems(ctx, cfg, newton_iters=newton_iters, model=model):
            b = sysm.residual.clone()
            res = {}
            for kind in ("jacobi", "learned"):
                x = torch.zeros_like(b)
                if kind == "learned":
                    net.attach(sysm.plan)
                else:
                    lpcg.use_block_jacobi(sysm.plan)
                torch.cuda.synchronize()
                t = time.perf_counter()
                rep = lpcg.plan_pcg(sysm.plan, sysm.values, b, x)
                torch.cuda.synchronize()
                res[kind] = (rep.iterations, bool(rep.converged), rep.rel_residual, time.perf_counter() - t)
            lpcg.use_block_jacobi(sysm.plan)
            row = dict(n=n, newton_iteration=sysm.meta["newton_iteration"], jacobi=res["jacobi"][0],
                       learned=res["learned"][0], converged=res["jacobi"][1] and res["learned"][1],
                       ratio=res["learned"][0] / max(res["jacobi"][0], 1),
                       seconds_jacobi=round(res["jacobi"][3], 4), seconds_learned=round(res["learned"][3], 4))
            out.append(row)
            log(json.dumps(row))
    return out


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--systems", type=int, default=48, help="Newton configurations to draw")
    ap.add_argument("--newton-iters", type=int, default=3)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--lr-end", type=float, default=1e-4)
    ap.add_argument("--probes", type=int, default=4)
    ap.add_argument("--nmin", type=int, default=8)
    ap.add_argument("--nmax", type=int, default=20)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--eval", default="14,24")
    ap.add_argument("--out", default=None)
    ap.add_argument("--init", default=None, help="start from these weights")
    ap.add_argument("--models", default="neohookean", help="comma-separated material models of the training cubes")
    ap.add_argument("--ratio", default="30,30000", help="range of E dt^2 / (rho h^2) of the training cubes")
    ap.add_argument("--nu", default="0.30,0.48", help="range of Poisson ratios")
    ap.add_argument("--stretch", type=float, default=0.15, help="initial per-axis stretch range 1 +- s")
    ap.add_argument("--kind", default="newton", choices=["newton", "rest", "stream"],
                    help="newton: Newton-iteration Hessians with residuals; rest: Hessians at perturbed rest states; "
                         "stream: Newton systems of packed batched-style instances, streamed through a rolling pool "
                         "(--systems counts instance systems)")
    ap.add_argument("--per-pack", type=int, default=16, help="stream: instances per packed plan")
    ap.add_argument("--pool", type=int, default=8, help="stream: packed systems held for sampling")
    ap.add_argument("--no-residual", action="store_true", help="train with Rademacher probes only")
    ap.add_argument("--hetero", type=float, default=0.0,
                    help="sigma of a log-normal per-tet stiffness factor on a fraction of the cubes")
    ap.add_argument("--hetero-frac", type=float, default=0.5, help="fraction of the cubes made heterogeneous")
    args = ap.parse_args(argv)
    import bartels_gb300 as bg
    from . import lpcg
    ctx = bg.Context.default()
    t0 = time.time()
    systems = []
    models = tuple(m for m in args.models.split(",") if m)
    rr = tuple(float(v) for v in args.ratio.split(","))
    nr = tuple(float(v) for v in args.nu.split(","))
    if args.kind == "stream":
        net = lpcg.LearnedPreconditioner.load(args.init, ctx) if args.init else lpcg.LearnedPreconditioner(
            ctx, seed=args.seed)
        hist, produced = lpcg.train_stream(net, ctx, args.systems, args.steps, per_pack=args.per_pack,
                                           n_range=(args.nmin, args.nmax), newton_iters=args.newton_iters,
                                           pool=args.pool, lr=args.lr, lr_end=args.lr_end, nprobes=args.probes,
                                           seed=args.seed, log=lambda s: print(s, flush=True))
        t_train = time.time() - t0
        print(f"stream training: {produced} instance systems, {len(hist)} steps in {t_train:.1f}s", flush=True)
        rows = evaluate(ctx, net, [int(s) for s in args.eval.split(",") if s])
        if args.out and hist:
            net.save(args.out, loss_first=np.mean(hist[:20]), loss_last=np.mean(hist[-50:]), steps=len(hist),
                     systems=produced, seed=args.seed, lr=args.lr, probes=args.probes, kind="stream",
                     eval_ratio=np.mean([r["ratio"] for r in rows]) if rows else np.nan)
            print("wrote", args.out, flush=True)
        return rows
    for cfg in lpcg.sample_configs(args.systems, seed=args.seed, n_range=(args.nmin, args.nmax), models=models,
                                   ratio_range=rr, nu_range=nr, stretch=args.stretch, hetero=args.hetero,
                                   hetero_frac=args.hetero_frac):
        cfg["seed"] = len(systems)
        if args.kind == "newton":
            systems += lpcg.newton_systems(ctx, cfg, newton_iters=args.newton_iters)
        else:
            systems += lpcg.perturbed_systems(ctx, cfg, count=args.newton_iters)
    t_data = time.time() - t0
    if args.systems:
        print(f"{len(systems)} systems from {args.systems} Newton runs in {t_data:.1f}s", flush=True)
    net = lpcg.LearnedPreconditioner.load(args.init, ctx) if args.init else lpcg.LearnedPreconditioner(ctx,
                                                                                                      seed=args.seed)
    t1 = time.time()
    hist = []
    if args.steps and systems:
        hist = lpcg.train(net, systems, args.steps, lr=args.lr, lr_end=args.lr_end, nprobes=args.probes,
                          seed=args.seed, log=lambda s: print(s, flush=True), residual_probe=not args.no_residual)
        t_train = time.time() - t1
        print(f"training: {args.steps} steps in {t_train:.1f}s ({1e3 * t_train / max(args.steps, 1):.2f} ms/step)",
              flush=True)
    sizes = [int(s) for s in args.eval.split(",") if s]
    rows = evaluate(ctx, net, sizes)
    if args.out and hist:
        net.save(args.out, loss_first=np.mean(hist[:20]), loss_last=np.mean(hist[-50:]), steps=args.steps,
                 systems=len(systems), seed=args.seed, lr=args.lr, probes=args.probes,
                 eval_ratio=np.mean([r["ratio"] for r in rows]) if rows else np.nan)
        print("wrote", args.out, flush=True)
    return rows


if __name__ == "__main__":
    main()
