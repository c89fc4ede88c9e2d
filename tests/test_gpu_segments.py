"""Packed meshes with per-instance semantics, through the C ABI.

With bartels_plan_set_segments the plan keeps one set of PCG scalars per
packed mesh and one line-search step per packed mesh, as the reference would
run one newtons_method_bisection (include/optimization_gradient_based.h:77-106)
with its own linesearch_backtracking_bisection
(src/linesearch_backtracking_bisection.cpp:17-30) per problem. The checks: a
packed mesh's PCG iteration count and Newton iterates do not depend on what it
is packed with (bit for bit, block-Jacobi preconditioner), the solutions match
each mesh solved alone, and inactive segments take no step."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _torch():
    return pytest.importorskip("torch")


def _instances(stiff_second):
    from bartels_gb300.batched import make_instances
    inst = make_instances(3, seed=7, n_range=(4, 7))
    inst[1] = dict(inst[1])
    if stiff_second:
        inst[1]["young"] = inst[1]["young"] * 1000.0  # a much stiffer neighbour
    return inst


def _packed_plan(inst, segments=True):
    import bartels_gb300 as bg
    from bartels_gb300 import _lib
    from bartels_gb300.api import volume
    from bartels_gb300.batched import pack
    pk = pack(inst)
    V, E = pk["V"], pk["E"]
    plan = bg.MeshPlan(V, E)
    plan.set_element_data(params=pk["params"], density=np.full(len(E), 1000.0))
    f_g = plan.const_ext_force(volume(V, E), np.array([0.0, 0.0, -9810.0]))
    plan.set_problem(q_base=pk["q_base"].ravel(), x_hat=np.zeros(3 * len(V)), f_ext=f_g, pinned=pk["pinned"])
    if segments:
        voff = np.ascontiguousarray(pk["voff"], np.int32)
        toff = np.ascontiguousarray(pk["toff"], np.int64)
        _lib.check(bg.lib().bartels_plan_set_segments(plan.handle, len(voff) - 1,
                                                      voff.ctypes.data_as(C.POINTER(C.c_int)),
                                                      toff.ctypes.data_as(C.POINTER(C.c_int64))), "segments")
    return plan, pk


def _hessian(plan, q):
    torch = _torch()
    import bartels_gb300 as bg
    from bartels_gb300 import _lib
    qd = torch.from_numpy(np.ascontiguousarray(q).ravel()).cuda()
    vals = torch.empty(plan.nnz, dtype=torch.float32, device="cuda")
    _lib.check(bg.lib().bartels_plan_hessian_d(plan.ctx.handle, plan.handle, _lib.NEOHOOKEAN, _lib.PSD_SIMPLE_FIX,
                                               1e-6, 0, 1e-4, 1.0, C.c_void_p(qd.data_ptr()),
                                               C.c_void_p(vals.data_ptr())), "hessian")
    plan.ctx.synchronize()
    return vals


def _seg_iters(plan, nseg):
    import bartels_gb300 as bg
    it = np.zeros(nseg, np.int32)
    bg.lib().bartels_plan_segment_pcg_iterations(plan.handle, it.ctypes.data_as(C.POINTER(C.c_int)))
    return it


def _solve(plan, vals, b):
    torch = _torch()
    from bartels_gb300 import lpcg
    lpcg.use_block_jacobi(plan)
    x = torch.zeros_like(b)
    rep = lpcg.plan_pcg(plan, vals, b, x, rel_tol=1e-8)
    assert rep.converged
    return x.cpu().numpy()


def test_a_stiff_neighbour_does_not_change_an_instance_pcg():
    torch = _torch()
    out = {}
    for stiff in (False, True):
        plan, pk = _packed_plan(_instances(stiff))
        vals = _hessian(plan, pk["q_base"])
        rng = np.random.default_rng(5)
        b = rng.standard_normal(3 * len(pk["V"]))
        b[np.repeat(pk["pinned"].astype(bool), 3)] = 0.0
        x = _solve(plan, vals, torch.from_numpy(b).cuda())
        out[stiff] = (x, _seg_iters(plan, len(pk["voff"]) - 1), pk["voff"])
        plan.close()
    (x0, it0, voff), (x1, it1, _) = out[False], out[True]
    a = slice(3 * voff[0], 3 * voff[1])
    c = slice(3 * voff[2], 3 * voff[3])
    # instances 0 and 2 are untouched by their neighbour's stiffness: same iterations, same solution bits
    assert it0[0] == it1[0] and it0[2] == it1[2], (it0, it1)
    assert np.array_equal(x0[a], x1[a]) and np.array_equal(x0[c], x1[c])
    assert it0[1] != it1[1]  # the stiff instance itself needs another count


def test_segmented_solve_matches_each_mesh_alone():
    torch = _torch()
    inst = _instances(True)
    plan, pk = _packed_plan(inst)
    vals = _hessian(plan, pk["q_base"])
    rng = np.random.default_rng(6)
    b = rng.standard_normal(3 * len(pk["V"]))
    b[np.repeat(pk["pinned"].astype(bool), 3)] = 0.0
    x = _solve(plan, vals, torch.from_numpy(b).cuda())
    plan.close()
    for k in range(len(inst)):
        solo, spk = _packed_plan([inst[k]], segments=False)
        sv = _hessian(solo, spk["q_base"])
        sl = slice(3 * pk["voff"][k], 3 * pk["voff"][k + 1])
        xs = _solve(solo, sv, torch.from_numpy(b[sl].copy()).cuda())
        assert np.linalg.norm(x[sl] - xs) <= 1e-6 * np.linalg.norm(xs), k
        solo.close()


def test_per_instance_newton_iterates_and_inactive_segments():
    torch = _torch()
    import bartels_gb300 as bg
    from bartels_gb300 import _lib, lpcg
    traj = {}
    for stiff in (False, True):
        plan, pk = _packed_plan(_instances(stiff))
        lpcg.use_block_jacobi(plan)
        prm = bg.newton_params(model="neohookean", psd_mode=_lib.PSD_SIMPLE_FIX, psd_tol=1e-6, mass_coeff=1.0,
                               scale=0.01, force_scale=0.01, gradient_tol=0.0, relative=0, max_iterations=100)
        x = torch.zeros(3 * len(pk["V"]), dtype=torch.float64, device="cuda")
        rep = _lib.NewtonReport()
        xs = []
        for _ in range(3):
            done = C.c_int()
            _lib.check(bg.lib().bartels_newton_iterate_d(plan.ctx.handle, plan.handle, C.byref(prm),
                                                         C.c_void_p(x.data_ptr()), C.c_double(1.0), C.byref(done),
                                                         C.byref(rep)), "newton_iterate")
            plan.ctx.synchronize()
            xs.append(x.cpu().numpy().copy())
        # freeze instance 0: it takes no further step
        act = np.array([0, 1, 1], np.uint8)
        _lib.check(bg.lib().bartels_plan_set_segment_active(plan.handle, act.ctypes.data_as(C.c_void_p)), "active")
        done = C.c_int()
        _lib.check(bg.lib().bartels_newton_iterate_d(plan.ctx.handle, plan.handle, C.byref(prm),
                                                     C.c_void_p(x.data_ptr()), C.c_double(1.0), C.byref(done),
                                                     C.byref(rep)), "newton_iterate")
        plan.ctx.synchronize()
        x4 = x.cpu().numpy()
        v = pk["voff"]
        assert np.array_equal(x4[3 * v[0]:3 * v[1]], xs[-1][3 * v[0]:3 * v[1]])
        assert not np.array_equal(x4[3 * v[1]:3 * v[2]], xs[-1][3 * v[1]:3 * v[2]])
        traj[stiff] = (xs, v)
        plan.close()
    (xa, v), (xb, _) = traj[False], traj[True]
    for k in range(3):
        # instance 0's Newton iterates do not depend on its neighbour: same bits
        assert np.array_equal(xa[k][3 * v[0]:3 * v[1]], xb[k][3 * v[0]:3 * v[1]]), k
