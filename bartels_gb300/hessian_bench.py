"""Time the fused FP32 Hessian assembly of a Kuhn cube at a few states, with and
without the PSD projection.

    python -m bartels_gb300.hessian_bench [--n 96] [--model neohookean] [--reps 10] [--psd on|off|both]

States (seeded): "rest" (q = X: every element passes the exact PSD test),
"stretch_noise" (X scaled by (0.9, 1.05, 1.0) plus vertex noise 0.05 h: most
elements are projected) and "gravity_like" (a small sag in z plus vertex noise
0.002 h: a fraction of the elements is projected). E = 2e6 Pa, nu = 0.45,
simple_psd_fix tol 1e-6 when the projection is on. Each entry gives
milliseconds per assembly (device time of `reps` back-to-back calls on the
library's stream, CUDA events) and the compulsory byte rate (tet inputs 64 B +
vertex positions 12 B + CSR values written 4 B each) with its fraction of the
measured HBM copy bandwidth.
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


def hbm_peak():
    """Measured HBM copy bandwidth (GB/s) from MEASURED_PEAKS.json at the repository root, else 6800."""
    import os
    try:
        with open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"])
    except Exception:
        return 6800.0


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=96)
    ap.add_argument("--model", default="neohookean")
    ap.add_argument("--reps", type=int, default=10)
    ap.add_argument("--psd", default="both", choices=["on", "off", "both"])
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
    peak = hbm_peak()
    modes = {"on": [("psd_on", _lib.PSD_SIMPLE_FIX)], "off": [("psd_off", _lib.PSD_NONE)],
             "both": [("psd_off", _lib.PSD_NONE), ("psd_on", _lib.PSD_SIMPLE_FIX)]}[args.psd]
    # CUDA events on the library's own stream
    stream = torch.cuda.ExternalStream(int(L.bartels_ctx_stream(ctx.handle)), device=f"cuda:{ctx.device}")
    out = {}
    for name, q in states(V, args.n).items():
        qd = torch.from_numpy(q.ravel().copy()).cuda()
        for tag, psd in modes:
            def f():
                _lib.check(L.bartels_plan_hessian_d(ctx.handle, plan.handle, model, psd, 1e-6, 0, 1.0, 0.0,
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
            gbs = compulsory / ms / 1e6
            out[f"{name}/{tag}"] = dict(ms=round(ms, 4), compulsory_gbs=round(gbs, 1),
                                        frac_of_measured_hbm=round(gbs / peak, 3))
    line = dict(n=args.n, model=args.model, tets=nT, vertices=nV, compulsory_bytes=compulsory,
                hbm_gbs=peak, states=out)
    print(json.dumps(line), flush=True)
    plan.close()
    return line


if __name__ == "__main__":
    main()
