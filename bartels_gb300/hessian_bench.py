"""Time the fused FP32 Hessian assembly (PSD-projected) of a Kuhn cube at a few states.

    python -m bartels_gb300.hessian_bench [--n 96] [--model neohookean] [--reps 10]

States (seeded): "rest" (q = X: every element passes the exact PSD test),
"stretch_noise" (X scaled by (0.9, 1.05, 1.0) plus vertex noise 0.05 h: most
elements are projected) and "gravity_like" (a small sag in z plus vertex noise
0.002 h: a fraction of the elements is projected). E = 2e6 Pa, nu = 0.45,
simple_psd_fix tol 1e-6. Each line gives milliseconds per assembly (device
time of `reps` back-to-back calls on the library's stream, CUDA events) and two
byte rates: compulsory (tet inputs 64 B + vertex positions 12 B + CSR values
written 4 B each) and algorithmic (the traffic of the two-kernel formulation:
element kernel 64 T + 12 V + 576 T written, reduction kernel 576 T read + 4 nnz
written + 576 T of scatter map).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json

import numpy as np


def states(V, n, seed=0):
    rng = np.random.default_rng(seed)
    h = 1.0 / n
    sag = np.stack([0 * V[:, 0], 0 * V[:, 1], -0.02 * V[:, 2] * (1 - V[:, 2])], 1)
    return {"rest": V,
            "stretch_noise": V * np.array([0.9, 1.05, 1.0]) + 0.05 * h * rng.uniform(-1, 1, V.shape),
            "gravity_like": V + sag + 0.002 * h * rng.uniform(-1, 1, V.shape)}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=96)
    ap.add_argument("--model", default="neohookean")
    ap.add_argument("--reps", type=int, default=10)
    args = ap.parse_args(argv)
    import torch
    import bartels_gb300 as bg
    from bartels_gb300 import _lib
    from bartels_gb300.meshes import kuhn_cube, material_params
    L = bg.lib()
    ctx = bg.Context.default()
    V, E = kuhn_cube(args.n)
    plan = bg.MeshPlan(V, E, ctx)
    plan.set_element_data(params=material_params(args.model, len(E), 2e6, 0.45))
    model = bg.api.MODELS[args.model]
    nT, nV, nnz = len(E), len(V), plan.nnz
    compulsory = 64 * nT + 12 * nV + 4 * nnz
    algorithmic = 64 * nT + 12 * nV + 576 * nT + 576 * nT + 4 * nnz + 4 * 144 * nT
    # CUDA events on the library's own stream
    stream = torch.cuda.ExternalStream(int(L.bartels_ctx_stream(ctx.handle)), device=f"cuda:{ctx.device}")
    out = {}
    for name, q in states(V, args.n).items():
        qd = torch.from_numpy(q.ravel().copy()).cuda()

        def f():
            _lib.check(L.bartels_plan_hessian_d(ctx.handle, plan.handle, model, _lib.PSD_SIMPLE_FIX, 1e-6, 0, 1.0, 0.0,
                                                C.c_void_p(qd.data_ptr()), None), "bartels_plan_hessian_d")
        for _ in range(3):
            f()
        ctx.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(args.reps):
            f()
        b.record(stream)
        ctx.synchronize()
        ms = a.elapsed_time(b) / args.reps
        out[name] = dict(ms=round(ms, 4), compulsory_gbs=round(compulsory / ms / 1e6, 1),
                         algorithmic_gbs=round(algorithmic / ms / 1e6, 1))
    line = dict(n=args.n, model=args.model, tets=nT, vertices=nV, compulsory_bytes=compulsory,
                algorithmic_bytes=algorithmic, states=out)
    print(json.dumps(line), flush=True)
    plan.close()
    return line


if __name__ == "__main__":
    main()
