"""Newton iterations per second on the n=96 Neo-Hookean Kuhn cube (5,308,416 tets).

Workload (one "step" = one Newton iteration): implicit Euler in velocity form
(dt = 0.01) from rest under gravity, z = 0 face pinned, Neo-Hookean E = 2e6 Pa,
nu = 0.45, rho = 1000, Hessians PSD-projected (simple_psd_fix, tol 1e-6), each
Newton system solved by PCG to 1e-8 relative residual (FP32 PCG; the residual
b - A x is recomputed to ~2^-48 (float-float) after each reduction of the
inner residual and CG continues against it), Newton to 1e-8 relative gradient
norm; when a time step converges the next one starts. Synthetic, seeded
inputs (no dataset).

The headline value is learned-preconditioned PCG: one aggregation-multigrid
V-cycle per PCG iteration whose finest-level smoother is the network's factor
M = G^T G, rebuilt from each Newton Hessian inside the timed region (weights
trained by bartels_gb300/train_lpcg.py on other cubes). Beside it, the same
workload is timed on the same GPU with the same V-cycle smoothed by
block-Jacobi, i.e. without the network ("multigrid_pcg_without_network"), and
with block-Jacobi PCG ("jacobi_pcg").

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                    [--precond learned_multigrid|multigrid|learned|jacobi]

Prints one JSON line. Under torchrun (N > 1) every rank runs an independent
replica on its own GPU and rank 0 reports the max-over-ranks time. The path
could shard (a vertex partition with a one-layer halo), but every run here has
one GPU, so the multi-GPU mode is replicas only, with no collective on the
data path.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Newton iters/s (5.3M-tet NH): learned-PCG vs Jacobi-PCG, same GB300, 1e-8 res"
UNIT = "Newton iters/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=6)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=96)
    ap.add_argument("--model", default="neohookean")
    ap.add_argument("--no-psd", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=1)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-faithful-baseline", action="store_true",
                    help="skip the 1-thread reference-structured CPU sample beside the OpenMP baseline")
    ap.add_argument("--precond", default="learned_multigrid",
                    choices=["learned_multigrid", "multigrid", "learned", "jacobi"])
    ap.add_argument("--config", default="cube", choices=["cube", "batched", "stress"],
                    help="cube: the n=96 Newton benchmark; batched: 256 packed uneven cubes, one implicit-Euler "
                         "step; stress: the carved heterogeneous cube under 50%% compression")
    ap.add_argument("--no-multigrid-arm", action="store_true",
                    help="skip the multigrid arm without the network beside a learned_multigrid headline")
    ap.add_argument("--weights", default=os.path.join(ROOT, "bartels_gb300", "weights", "lpcg_neohookean.npz"))
    ap.add_argument("--no-jacobi-arm", action="store_true", help="skip the block-Jacobi comparison run")
    ap.add_argument("--no-autotune", action="store_true", help="default lane counts instead of the autotuner's")
    return ap.parse_args()


# ------------------------------------------------------------------ setup ---
def build_problem(n, model, seed=0):
    from bartels_gb300.meshes import kuhn_cube, material_params
    V, E = kuhn_cube(n)
    rho, young, nu, dt = 1000.0, 2e6, 0.45, 0.01
    params = material_params(model, len(E), young, nu)
    pinned = np.zeros(len(V), np.uint8)
    pinned[np.abs(V[:, 2] - V[:, 2].min()) <= 1e-9] = 1
    return dict(V=V, E=E, rho=rho, dt=dt, params=params, pinned=pinned,
                gravity=np.array([0.0, 0.0, -9.81]))


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = max(mx, float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------- replicas -------
def reduce_max_ms(ms, world, device="cpu"):
    """Max over ranks of the timed region (ms); identity for one process."""
    if world <= 1:
        return ms
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replica_value(newton_its_per_rank, world, ms):
    """Whole-job Newton iterations per second: every replica runs the same
    number of iterations; the job takes as long as the slowest replica."""
    return newton_its_per_rank * world / (ms * 1e-3)


# ------------------------------------------------------------ GPU arm ---------
def run_gpu(args, rank, world):
    import torch
    import bartels_gb300 as bg
    from bartels_gb300 import _lib

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    L = bg.lib()
    ctx = bg.Context(dev)
    stream = torch.cuda.ExternalStream(int(L.bartels_ctx_stream(ctx.handle)), device=f"cuda:{dev}")
    pb = build_problem(args.n, args.model)
    V, E = pb["V"], pb["E"]
    nV, nT = len(V), len(E)
    t0 = time.time()
    plan = bg.MeshPlan(V, E, ctx)
    t_plan = time.time() - t0
    density = np.full(nT, pb["rho"])
    plan.set_element_data(params=pb["params"], density=density)
    f_g = plan.const_ext_force(None, pb["rho"] * pb["gravity"])
    qt = V.ravel().copy()
    vt = np.zeros(3 * nV)
    plan.set_problem(q_base=qt, x_hat=vt, f_ext=f_g, pinned=pb["pinned"])
    psd = _lib.PSD_NONE if args.no_psd else _lib.PSD_SIMPLE_FIX
    prm = bg.newton_params(model=args.model, psd_mode=psd, psd_tol=1e-6, gradient_tol=1e-8, relative=1,
                           mass_coeff=1.0, scale=pb["dt"], force_scale=pb["dt"], max_iterations=100)
    x = torch.zeros(3 * nV, dtype=torch.float64, device=f"cuda:{dev}")
    xp = C.c_void_p(x.data_ptr())
    # lane counts of the SpMV and factor passes from the library's autotuner (plan setup,
    # outside the timed region), on the Hessian of the rest state
    lanes = None
    if not args.no_autotune:
        hv = torch.empty(plan.nnz, dtype=torch.float32, device=f"cuda:{dev}")
        q0 = torch.from_numpy(qt).to(f"cuda:{dev}")
        torch.cuda.synchronize()  # x and q0 written on torch's stream before the library reads them
        # assembly CTA shape and PSD pre-pass block size (values do not depend on them)
        h_c, h_b = C.c_int(), C.c_int()
        _lib.check(L.bartels_plan_autotune_hessian(ctx.handle, plan.handle, bg.api.MODELS[args.model],
                                                   C.c_void_p(q0.data_ptr()), 0, C.byref(h_c), C.byref(h_b)),
                   "autotune_hessian")
        _lib.check(L.bartels_plan_hessian_d(ctx.handle, plan.handle, bg.api.MODELS[args.model], psd, 1e-6, 0,
                                            pb["dt"] ** 2, 1.0, C.c_void_p(q0.data_ptr()), C.c_void_p(hv.data_ptr())),
                   "hessian")
        a_l, b_l = C.c_int(), C.c_int()
        _lib.check(L.bartels_plan_autotune(ctx.handle, plan.handle, C.c_void_p(hv.data_ptr()), 0, C.byref(a_l),
                                           C.byref(b_l)), "autotune")
        lanes = {"spmv": a_l.value, "factor": b_l.value, "hessian_chunk_vertices": h_c.value,
                 "psd_block": h_b.value}
        del hv, q0
    net = None
    if args.precond in ("learned", "learned_multigrid"):
        from bartels_gb300 import lpcg
        net = lpcg.LearnedPreconditioner.load(args.weights, ctx)

    def set_precond(kind):
        # multigrid solves converge in few iterations: a 100x residual reduction per refinement pass
        # (10x passes are the block-Jacobi and factor setting, which needs them against FP32 drift)
        prm.pcg.inner_rel_tol = 1e-2 if kind in ("multigrid", "learned_multigrid") else 1e-1
        if kind == "learned":
            net.attach(plan)
        elif kind == "learned_multigrid":
            net.attach(plan, multigrid=True)
        elif kind == "multigrid":
            _lib.check(L.bartels_plan_set_preconditioner(plan.handle, _lib.PRECOND_MULTIGRID, None), "precond")
        else:
            _lib.check(L.bartels_plan_set_preconditioner(plan.handle, _lib.PRECOND_BLOCK_JACOBI, None), "precond")

    def timed_newton(kind):
        """W warm-up and K timed Newton iterations from rest (fresh state)."""
        set_precond(kind)
        plan.set_problem(q_base=qt, x_hat=vt, f_ext=f_g, pinned=pb["pinned"])
        x.zero_()
        state = {"g0": -1.0, "steps": 0, "floor": 0}
        rep = _lib.NewtonReport()

        def newton_step():
            """Run until one Newton iteration (Hessian + PCG + line search) completed.
            A time step ends when the relative gradient test passes, or when the
            line search found no decrease at all (every trial rejected): the
            step has reached the rounding floor of its FP64 gradient, which on
            this system lies near the 1e-8 criterion, and further iterations
            cannot move it (the reference's loop would spin to its cap)."""
            while True:
                done = C.c_int()
                ls_fail = rep.ls_failures
                _lib.check(L.bartels_newton_iterate_d(ctx.handle, plan.handle, C.byref(prm), xp, state["g0"],
                                                      C.byref(done), C.byref(rep)), "newton_iterate")
                if state["g0"] < 0:
                    state["g0"] = rep.grad_norm
                if not done.value and rep.ls_failures > ls_fail:
                    state["floor"] += 1
                    done.value = 1
                if done.value:
                    # converged time step: q_t += dt v, v_t = v; next step starts from v
                    _lib.check(L.bartels_newton_advance_implicit_euler_d(ctx.handle, plan.handle, pb["dt"], xp),
                               "advance")
                    state["g0"] = -1.0
                    state["steps"] += 1
                    continue
                return

        for _ in range(args.warmup):
            newton_step()
        ctx.synchronize()
        before = (rep.iterations, rep.pcg_iterations, rep.ls_iterations, rep.precond_fallbacks, rep.t_precond)
        launches0 = ctx.kernel_launches
        if world > 1:
            torch.distributed.barrier()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with Clocks(dev) as clk:
            ctx.synchronize()
            ev0.record(stream)
            for _ in range(args.steps):
                newton_step()
            ev1.record(stream)
            ctx.synchronize()
            torch.cuda.synchronize()
        ms = reduce_max_ms(ev0.elapsed_time(ev1), world, f"cuda:{dev}")
        return dict(ms=ms, launches=ctx.kernel_launches - launches0, clocks=clk.summary(), rep=rep,
                    newton_its=rep.iterations - before[0], pcg_its=rep.pcg_iterations - before[1],
                    ls_its=rep.ls_iterations - before[2], fallbacks=rep.precond_fallbacks - before[3],
                    t_precond=rep.t_precond - before[4], steps=state["steps"], g0=state["g0"],
                    steps_at_noise_floor=state["floor"])

    def oracle_check(cw, arm):
        """The FP64 oracle (CPU restatement) against the GPU at the state after the
        timed iterations: the Newton objective's energy and gradient there; then
        the time step is finished on the GPU (untimed) and the oracle's gradient
        at its solution, relative to the step's initial gradient, is the
        solution's error against the 1e-8 criterion."""
        Dp = C.POINTER(C.c_double)
        qb, xh = np.zeros(3 * nV), np.zeros(3 * nV)
        _lib.check(L.bartels_newton_get_problem(plan.handle, qb.ctypes.data_as(Dp), xh.ctypes.data_as(Dp)), "state")
        cw.set_state(qb, xh)
        xs = x.cpu().numpy()
        e_gpu = C.c_double()
        _lib.check(L.bartels_newton_energy_d(ctx.handle, plan.handle, C.byref(prm), xp, C.byref(e_gpu)), "energy")
        g_gpu = torch.empty_like(x)
        _lib.check(L.bartels_newton_gradient_d(ctx.handle, plan.handle, C.byref(prm), xp,
                                               C.c_void_p(g_gpu.data_ptr())), "gradient")
        ctx.synchronize()  # the library's stream, not torch's
        gg = g_gpu.cpu().numpy()
        e_cpu, g_cpu = cw.cb.energy(xs), cw.cb.gradient(xs)
        g0 = arm["g0"] if arm["g0"] > 0 else float(np.linalg.norm(gg))
        # the gradient error relative to the step's initial gradient g0 (near
        # convergence the gradient itself is a ~1e-8 g0 remainder of cancelling
        # element forces, and its error relative to its own norm is rounding noise)
        out = {"state": f"after the timed iterations (time step {arm['steps'] + 1} of the run, mid-solve)",
               "energy_rel_err": abs(e_gpu.value - e_cpu) / abs(e_cpu),
               "gradient_err_rel_g0": float(np.linalg.norm(gg - g_cpu) / g0),
               "gradient_norm_rel_g0": float(np.linalg.norm(g_cpu) / g0)}
        its, rep2, trace = 0, _lib.NewtonReport(), []
        floor = False
        while its < 40:
            done = C.c_int()
            _lib.check(L.bartels_newton_iterate_d(ctx.handle, plan.handle, C.byref(prm), xp, g0, C.byref(done),
                                                  C.byref(rep2)), "newton_iterate")
            trace.append({"rel_grad": rep2.grad_norm / g0, "alpha": rep2.last_alpha,
                          "pcg": rep2.last_pcg_iterations, "pcg_rel_res": rep2.last_pcg_rel_residual})
            if done.value:
                break
            its += 1
            if rep2.ls_failures > 0:  # no decrease found: the FP64 rounding floor
                floor = True
                break
        ctx.synchronize()
        g_sol = cw.cb.gradient(x.cpu().numpy())
        out["time_step_solution"] = {"newton_iterations_to_finish": its, "criterion": 1e-8, "converged": bool(done.value),
                                     "ended_at_noise_floor": floor,
                                     "fp64_relative_gradient": float(np.linalg.norm(g_sol) / g0),
                                     "trace": trace[-6:]}
        return out

    main_arm = timed_newton(args.precond)
    mg_levels = None
    if args.precond in ("multigrid", "learned_multigrid"):
        from bartels_gb300 import lpcg
        mg_levels = lpcg.mg_info(plan)
    cpu_work, oracle_err = None, None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu_work = CpuWorkload(pb, args)
        oracle_err = oracle_check(cpu_work, main_arm)
    mg_arm = timed_newton("multigrid") if (args.precond == "learned_multigrid" and not args.no_multigrid_arm) else None
    jac = main_arm if args.precond == "jacobi" else (None if args.no_jacobi_arm else timed_newton("jacobi"))
    L.bartels_plan_set_preconditioner(plan.handle, _lib.PRECOND_BLOCK_JACOBI, None)
    ms, launches, rep = main_arm["ms"], main_arm["launches"], main_arm["rep"]
    pcg_its, newton_its = main_arm["pcg_its"], main_arm["newton_its"]
    state = {"steps": main_arm["steps"]}

    # --- roofline of the dominant kernel (PCG SpMV) and the dq2 assembly, live
    n_dof = 3 * nV
    xs = torch.randn(n_dof, dtype=torch.float32, device=f"cuda:{dev}")
    ys = torch.empty_like(xs)
    torch.cuda.synchronize()  # torch's stream before the library's
    nnz = plan.nnz
    nnzb = nnz // 9

    def time_launch(fn, reps):
        for _ in range(2):
            fn()
        ctx.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(reps):
            fn()
        b.record(stream)
        ctx.synchronize()
        return a.elapsed_time(b) / reps * 1e-3

    # the PCG loop's own SpMV kernel (over the padded copy of the values the loop
    # reads), timed by the library with CUDA events on its stream
    spmv_us = C.c_double()
    _lib.check(L.bartels_plan_pcg_spmv_time_d(ctx.handle, plan.handle, None, C.c_void_p(xs.data_ptr()),
                                              C.c_void_p(ys.data_ptr()), 30, C.byref(spmv_us)), "pcg_spmv_time")
    spmv_s = spmv_us.value * 1e-6
    spmv_bytes = 4 * nnz + 4 * nnzb + 4 * (nV + 1) + 12 * nV + 12 * nV
    qd = torch.from_numpy(V.ravel().copy()).to(f"cuda:{dev}")
    torch.cuda.synchronize()
    model_id = bg.api.MODELS[args.model]

    def hess_time(psd_mode):
        return time_launch(lambda: _lib.check(L.bartels_plan_hessian_d(ctx.handle, plan.handle, model_id, psd_mode,
                                                                       1e-6, 0, 1.0, 0.0, C.c_void_p(qd.data_ptr()),
                                                                       None), "hess"), 5)
    hess_off_s = hess_time(_lib.PSD_NONE)
    hess_on_s = hess_time(_lib.PSD_SIMPLE_FIX)
    # dq2 compulsory bytes (n=96: 0.84 GB): tet records (64 B) + vertex positions
    # (12 B) + CSR values written (4 B each)
    hess_bytes = 64 * nT + 12 * nV + 4 * nnz
    peak, peak_kind = peaks()
    spmv_gbs = spmv_bytes / spmv_s / 1e9
    traffic = None
    try:
        with open(os.path.join(ROOT, "profiles", "spmv_traffic.json")) as f:
            tj = json.load(f)
        # DRAM bytes per launch from one ncu capture of a smaller cube, scaled by the
        # algorithmic bytes (the SpMV's traffic grows in proportion to its nnz)
        traffic = float(tj["ratio"]) * spmv_bytes
    except Exception:
        pass

    # --- end to end through the host-buffer public API (one implicit-Euler step per e2e step)
    e2e = None
    if rank == 0 and args.e2e_steps > 0:
        plan.set_problem(q_base=qt, x_hat=vt, f_ext=f_g, pinned=pb["pinned"])
        set_precond(args.precond)
        v_host = np.zeros(3 * nV)
        its = 0
        t = 0.0
        h2d = d2h = 0
        for _ in range(args.e2e_steps):
            t1 = time.perf_counter()
            v_out, r = plan.newton_solve(v_host, prm)
            t += time.perf_counter() - t1
            its += r.iterations
            h2d += v_host.nbytes
            d2h += v_out.nbytes
        # the same solves with the state already on the device: the window differs
        # from `value`'s (whole time steps from rest here), so this is the figure
        # the host copies are measured against
        vd = torch.zeros(3 * nV, dtype=torch.float64, device=f"cuda:{dev}")
        its_d, t_d = 0, 0.0
        for _ in range(args.e2e_steps):
            vd.zero_()
            torch.cuda.synchronize()
            rd = _lib.NewtonReport()
            t1 = time.perf_counter()
            _lib.check(L.bartels_newton_solve_d(ctx.handle, plan.handle, C.byref(prm), C.c_void_p(vd.data_ptr()),
                                                C.byref(rd)), "bartels_newton_solve_d")
            ctx.synchronize()
            t_d += time.perf_counter() - t1
            its_d += rd.iterations
        L.bartels_plan_set_preconditioner(plan.handle, _lib.PRECOND_BLOCK_JACOBI, None)
        e2e = {"value": its / t if t > 0 else None, "unit": UNIT,
               "h2d_bytes_per_step": h2d // args.e2e_steps, "d2h_bytes_per_step": d2h // args.e2e_steps,
               "newton_iterations": its, "seconds": t,
               "window": f"{args.e2e_steps} implicit-Euler step(s) from rest through bartels_newton_solve",
               "device_resident_same_window": its_d / t_d if t_d > 0 else None}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        # one whole Newton iteration of this workload (the first from rest) on the host cores, measured
        cw = cpu_work if cpu_work is not None else CpuWorkload(pb, args)
        cw.set_state(V.ravel().copy(), np.zeros(3 * nV))
        cw.x[:] = 0.0
        cw.g0 = -1.0
        t1 = time.perf_counter()
        st = cw.newton_step()
        t_one = time.perf_counter() - t1
        cpu = {"value": 1.0 / t_one, "unit": UNIT, "cores": cw.cb.threads, "kind": "port", "estimated": False,
               "sample": f"one whole Newton iteration of this workload (the first from rest), measured: FP64 OpenMP "
                         f"CPU restatement, gradient, simple_psd_fix Hessian over all {nT} tets, block-Jacobi PCG to "
                         f"1e-8 ({int(st['pcg_iterations'])} iterations), the reference's line search",
               "components": {k: st[k] for k in ("t_gradient", "t_hessian", "t_pcg", "t_linesearch")},
               "pcg_iterations": int(st["pcg_iterations"])}
        if not args.no_faithful_baseline:
            f_est, f_parts, f_scale = cpu_faithful_sample(pb, args, st["pcg_iterations"])
            cpu["reference_faithful_1thread"] = {
                "value": 1.0 / f_est, "unit": UNIT, "cores": 1, "estimated": True, "scales": f_scale,
                "sample": "ESTIMATE of one Newton iteration in the reference's structure on 1 thread (dense per-tet "
                          "B^T d2psi B + simple_psd_fix, triplets + sort/compress, serial sums) from 1/64 of the "
                          "tets x64 and 3 one-thread PCG iterations scaled to the measured CPU PCG count",
                "components": f_parts}
    if cpu_work is not None:
        cpu_work.close()

    precond_name = {"learned": "learned factor G^T G", "jacobi": "block-Jacobi", "multigrid": "aggregation multigrid",
                    "learned_multigrid": "aggregation multigrid with the learned smoother"}[args.precond]
    value = replica_value(newton_its, world, ms)
    jacobi_pcg = None
    if jac is not None and args.precond != "jacobi":
        jv = replica_value(jac["newton_its"], world, jac["ms"])
        jacobi_pcg = {"value": jv, "unit": UNIT, "ms_per_step": jac["ms"] / max(jac["newton_its"], 1),
                      "pcg_iters_per_newton": jac["pcg_its"] / max(jac["newton_its"], 1),
                      "ls_backtracks_per_newton": jac["ls_its"] / max(jac["newton_its"], 1),
                      "newton_iterations": jac["newton_its"], "clocks": jac["clocks"],
                      "learned_over_jacobi": value / jv if jv > 0 else None}
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / max(newton_its, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic (seeded Kuhn cube, gravity)",
        "config": {"workload": f"implicit-Euler Newton, Neo-Hookean Kuhn cube n={args.n} "
                               f"({nV} vertices, {nT} tets), dt=0.01, z=0 pinned, PSD "
                               f"{'off' if args.no_psd else 'simple_psd_fix 1e-6'}, {precond_name} PCG 1e-8, "
                               "Newton 1e-8 relative", "preconditioner": precond_name,
                   "learned_pcg_weights": os.path.relpath(args.weights, ROOT) if net is not None else None,
                   "parallelism": f"replicas x{world}", "lanes_per_row": lanes,
                   "l2": "inputs larger than L2 (CSR values %.0f MB)" % (4 * nnz / 1e6)},
        "newton_iterations": newton_its, "pcg_iterations": pcg_its,
        "time_steps_ended_at_noise_floor": main_arm["steps_at_noise_floor"],
        "pcg_iters_per_newton": pcg_its / max(newton_its, 1),
        "roofline": {"bound": "hbm", "achieved": spmv_gbs, "peak": peak, "unit": "GB/s",
                     "frac": spmv_gbs / peak, "traffic": traffic, "kernel": "k_pcg_spmv_blk (the PCG loop's SpMV, FP32, rows padded to 4 entries)",
                     "bytes_per_launch": spmv_bytes, "us_per_launch": spmv_s * 1e6, "peak_source": peak_kind},
        "kernels": {"dq2_psd_off": {"us_per_launch": hess_off_s * 1e6, "state": "rest (q = X)",
                                    "compulsory_bytes": hess_bytes, "achieved_gbs": hess_bytes / hess_off_s / 1e9,
                                    "frac": hess_bytes / hess_off_s / 1e9 / peak, "bound": "hbm"},
                    "dq2_psd_on": {"us_per_launch": hess_on_s * 1e6, "state": "rest (q = X)",
                                   "compulsory_bytes": hess_bytes, "achieved_gbs": hess_bytes / hess_on_s / 1e9,
                                   "frac": hess_bytes / hess_on_s / 1e9 / peak}},
        "jacobi_pcg": jacobi_pcg,
        "multigrid_pcg_without_network": None if mg_arm is None else {
            "value": replica_value(mg_arm["newton_its"], world, mg_arm["ms"]), "unit": UNIT,
            "ms_per_step": mg_arm["ms"] / max(mg_arm["newton_its"], 1),
            "pcg_iters_per_newton": mg_arm["pcg_its"] / max(mg_arm["newton_its"], 1),
            "newton_iterations": mg_arm["newton_its"], "clocks": mg_arm["clocks"],
            "setup_ms_per_newton": 1e3 * mg_arm["t_precond"] / max(mg_arm["newton_its"], 1)},
        "learned_precond": None if args.precond == "jacobi" else {
            "factor_build_ms_per_newton": 1e3 * main_arm["t_precond"] / max(newton_its, 1),
            "fallbacks_to_block_jacobi": main_arm["fallbacks"],
            "pcg_us_per_iteration": 1e6 * rep.t_pcg / max(rep.pcg_iterations, 1)},
        "clocks": main_arm["clocks"], "gpu_launches": int(launches), "e2e": e2e, "cpu_baseline": cpu,
        "oracle_error": oracle_err, "multigrid_hierarchy": mg_levels,
        "setup_s": {"plan": t_plan}, "time_steps_completed": state["steps"],
        "stage_seconds": {"gradient": rep.t_gradient, "hessian": rep.t_hessian, "pcg": rep.t_pcg,
                          "linesearch": rep.t_linesearch},
    }
    return out


# --------------------------------------------------------- CPU baseline ----
class CpuWorkload:
    """The bench workload on the FP64 OpenMP CPU restatement of the path
    (oracle/oracle_baseline.cpp): implicit-Euler Newton from rest with the same
    state machine as the GPU arm (a converged time step advances q_base += dt v,
    x_hat = v, and the next step starts from v). Each Newton iteration is the
    reference's (include/optimization_gradient_based.h:77-106): gradient, the
    simple_psd_fix-projected Hessian over all tets, the search direction (block-
    Jacobi PCG to 1e-8 relative residual in place of Eigen::SparseLU, which
    cannot factor 2.7M DOF here) and the backtracking line search
    (src/linesearch_backtracking_bisection.cpp:17-30)."""

    def __init__(self, pb, args):
        from oracle import oracle as o
        from oracle.baseline import CpuNewton
        V, E = pb["V"], pb["E"]
        self.pb, self.args = pb, args
        self.cb = CpuNewton(V, E)
        self.f_g = o.const_ext_force(len(V), E, o.volume(V, E), pb["rho"] * pb["gravity"])
        self.q_base, self.x_hat = V.ravel().copy(), np.zeros(3 * len(V))
        self.x = np.zeros(3 * len(V))
        self.g0, self.steps = -1.0, 0
        self.set_state(self.q_base, self.x_hat)

    def set_state(self, q_base, x_hat):
        pb, a = self.pb, self.args
        self.q_base, self.x_hat = q_base, x_hat
        self.cb.set(a.model, pb["params"], np.full(len(pb["E"]), pb["rho"]), q_base, x_hat, self.f_g, pb["pinned"],
                    1.0, pb["dt"], pb["dt"], None if a.no_psd else 1e-6)

    def newton_step(self):
        """One whole Newton iteration (converged time steps are advanced first)."""
        while True:
            gn = float(np.linalg.norm(self.cb.gradient(self.x)))
            if self.g0 < 0:
                self.g0 = gn
            if gn > 1e-8 * self.g0:
                break
            self.set_state(self.q_base + self.pb["dt"] * self.x, self.x.copy())
            self.g0, self.steps = -1.0, self.steps + 1
        return self.cb.newton_iteration(self.x, 1e-8, 60000, 100)

    def close(self):
        self.cb.close()


def cpu_faithful_sample(pb, args, pcg_per_newton):
    """An ESTIMATE of one Newton iteration in the reference's own structure on one
    host thread, from bounded samples: per-tet dense B^T d2psi B with
    simple_psd_fix (tridiagonal QL, as Eigen's solver), a triplet list and a
    sort / compress into CSR (src/assemble.cpp:57-94), over 1/64 of the tets
    (x64); serial gradient and energy over the same slice (x64); the line
    search's two energy evaluations per trial
    (src/linesearch_backtracking_bisection.cpp:21); 3 block-Jacobi PCG
    iterations on the full system with one thread, scaled to the measured CPU
    PCG count per Newton iteration. Returns (seconds, components, scales)."""
    from oracle import oracle as o
    from oracle.baseline import CpuNewton, faithful_dq2
    V, E = pb["V"], pb["E"]
    nV, nT = len(V), len(E)
    sub = E[: max(1, nT // 64)]
    scale = nT / len(sub)
    q = V.ravel().copy()
    dphi, vol = o.dphi_dX(V, sub), o.volume(V, sub)
    params = pb["params"][: len(sub)]
    psd = None if args.no_psd else 1e-6
    t = time.perf_counter(); faithful_dq2(args.model, nV, sub, q, dphi, vol, params, psd)
    t_h = (time.perf_counter() - t) * scale
    t = time.perf_counter(); o.tetmesh_dq(args.model, nV, sub, q, dphi, vol, params)
    t_g = (time.perf_counter() - t) * scale
    t = time.perf_counter(); o.tetmesh_q(args.model, sub, q, dphi, vol, params)
    t_e = (time.perf_counter() - t) * scale
    cb = CpuNewton(V, E)
    cb.set(args.model, pb["params"], np.full(nT, pb["rho"]), q, np.zeros(3 * nV),
           o.const_ext_force(nV, E, o.volume(V, E), pb["rho"] * pb["gravity"]), pb["pinned"], 1.0, pb["dt"],
           pb["dt"], psd)
    threads = cb.threads
    x = np.zeros(3 * nV)
    g = cb.gradient(x)
    cb.hessian_range(x, 0, len(sub), True)  # PCG cost per iteration does not depend on the values
    cb.set_threads(1)
    try:
        d = np.zeros(3 * nV)
        t = time.perf_counter(); it, _ = cb.pcg(-g, d, 1e-30, 3); t_p = (time.perf_counter() - t) / max(it, 1)
    finally:
        cb.set_threads(threads)
        cb.close()
    est = t_g + t_h + pcg_per_newton * t_p + 2.0 * t_e
    return est, {"gradient_s": t_g, "hessian_s": t_h, "pcg_iter_s": t_p, "energy_s": t_e}, \
        {"tets_sampled": len(sub), "tet_scale": scale, "pcg_iterations_sampled": 3,
         "pcg_scale_to": pcg_per_newton}


def run_reference(args):
    """--impl reference: the reference's CPU path of this workload on the host
    cores (its FP64 restatement: the reference itself needs Eigen and libigl,
    absent here). Every timed step is one whole Newton iteration, measured:
    nothing is sampled or scaled. The W warm-up steps are gradient and energy
    evaluations (the first also assembles the Hessian), which touch every
    array a Newton iteration uses."""
    pb = build_problem(args.n, args.model)
    t0 = time.perf_counter()
    cw = CpuWorkload(pb, args)
    t_setup = time.perf_counter() - t0
    for w in range(args.warmup):
        cw.cb.gradient(cw.x)
        cw.cb.energy(cw.x)
        if w == 0:
            cw.cb.hessian_range(cw.x, 0, len(pb["E"]), True)
    secs, pcg, ls = [], [], []
    comp = {"t_gradient": 0.0, "t_hessian": 0.0, "t_pcg": 0.0, "t_linesearch": 0.0}
    for _ in range(max(args.steps, 1)):
        t = time.perf_counter()
        st = cw.newton_step()
        secs.append(time.perf_counter() - t)
        pcg.append(st["pcg_iterations"])
        ls.append(st["ls_iterations"])
        for k in comp:
            comp[k] += st[k]
    total = sum(secs)
    value = len(secs) / total
    threads = cw.cb.threads
    steps_done = cw.steps
    cw.close()
    return {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * total / len(secs), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Kuhn cube, gravity)",
            "config": {"workload": f"implicit-Euler Newton, Neo-Hookean Kuhn cube n={args.n}, dt=0.01, z=0 pinned, "
                                   f"PSD {'off' if args.no_psd else 'simple_psd_fix 1e-6'}, block-Jacobi PCG 1e-8, "
                                   "Newton 1e-8 relative", "parallelism": f"OpenMP host, {threads} threads"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{len(secs)} whole Newton iterations of the workload from rest, each measured "
                                       "(gradient, simple_psd_fix Hessian over all tets, block-Jacobi PCG to 1e-8, "
                                       "line search), FP64 OpenMP CPU restatement",
                             "estimated": False},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "pcg_iters_per_newton": float(np.mean(pcg)), "ls_backtracks_per_newton": float(np.mean(ls)),
            "seconds_per_step": secs, "stage_seconds": comp, "time_steps_completed": steps_done,
            "setup_s": t_setup}


def run_batched(args):
    """256 packed Neo-Hookean cubes (n uniform in [8, 40], E log-uniform in
    [1e5, 1e7], nu in [0.30, 0.48], per-axis stretch in [0.7, 1.3], noise
    0.01 h; seeds fixed), one implicit-Euler step, every instance to 1e-8
    relative gradient with its own PCG scalars and line-search step. Timed
    per preconditioner on the same GPU; value = tets x Newton iterations per
    second of the headline (learned multigrid)."""
    import bartels_gb300 as bg
    from bartels_gb300 import batched, lpcg
    inst = batched.make_instances(256, 0, (8, 40))
    packed = batched.pack(inst)
    net = lpcg.LearnedPreconditioner.load(args.weights, bg.Context.default())
    arms = {}
    for pc in ("learned_multigrid", "multigrid", "jacobi"):
        stats, rel, _ = batched.solve(packed, tol=1e-8, precond=pc, net=net, max_newton=100)
        arms[pc] = stats
    h = arms["learned_multigrid"]
    return {"metric": "tet-Newton iterations/s: 256 packed NH cubes n in [8,40], one implicit-Euler step, "
                      "each instance to 1e-8 relative gradient", "value": h["tets_x_newton_per_s"],
            "unit": "tet-Newton iters/s", "n_gpus": 1, "higher_is_better": True, "dtype": "f32+f64",
            "data": "synthetic (seeded packed Kuhn cubes)", "config": {"workload": "batched", "instances": 256,
                                                                       "vertices": h["vertices"], "tets": h["tets"]},
            "arms": arms, "learned_over_jacobi_seconds": arms["jacobi"]["seconds"] / h["seconds"]}


def run_stress(args):
    """The carved heterogeneous n=64 cube (log-normal E, 100x inclusions, nu
    0.47) under 50% axial compression in 10 load steps, each preconditioner on
    the same GPU."""
    import bartels_gb300 as bg
    from bartels_gb300 import lpcg, stress_case
    prob = stress_case.build(64, 0)
    net = lpcg.LearnedPreconditioner.load(args.weights, bg.Context.default())
    arms = {}
    for pc in ("learned_multigrid", "multigrid", "jacobi"):
        _, tot, _ = stress_case.run(prob, pc, net, steps=10, log=lambda s: None)
        arms[pc] = tot
    h = arms["learned_multigrid"]
    return {"metric": "Newton iterations/s: carved heterogeneous n=64 cube, 50% compression in 10 load steps",
            "value": h["newton"] / h["seconds"], "unit": "Newton iters/s", "n_gpus": 1, "higher_is_better": True,
            "dtype": "f32+f64", "data": "synthetic (seeded carving and materials)",
            "config": {"workload": "stress", "vertices": len(prob["V"]), "tets": len(prob["E"])}, "arms": arms,
            "learned_over_jacobi_seconds": arms["jacobi"]["seconds"] / h["seconds"]}


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.config != "cube" and args.impl != "reference":
        print(json.dumps(run_batched(args) if args.config == "batched" else run_stress(args)))
        return
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference(args)))
        return
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    out = run_gpu(args, rank, world)
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
