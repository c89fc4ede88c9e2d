"""Batched solves (many meshes packed into one plan): the per-mesh squared
norms, the autotuner, and batched implicit-Euler steps against the same meshes
solved one by one."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_segment_sumsq_matches_numpy():
    torch = pytest.importorskip("torch")
    import bartels_gb300 as bg
    from bartels_gb300 import _lib
    ctx = bg.Context.default()
    rng = np.random.default_rng(0)
    off = np.array([0, 5, 5, 130, 131, 1000], np.int32)
    v = rng.standard_normal(3 * off[-1])
    out = torch.empty(len(off) - 1, dtype=torch.float64, device="cuda")
    od, vd = torch.from_numpy(off).cuda(), torch.from_numpy(v).cuda()
    _lib.check(bg.lib().bartels_segment_sumsq_d(ctx.handle, len(off) - 1, C.c_void_p(od.data_ptr()),
                                                C.c_void_p(vd.data_ptr()), C.c_void_p(out.data_ptr())), "sumsq")
    ref = np.array([np.sum(v[3 * off[s]:3 * off[s + 1]] ** 2) for s in range(len(off) - 1)])
    assert np.allclose(out.cpu().numpy(), ref, rtol=1e-12, atol=0)


def test_autotuner_picks_valid_lanes_and_caches_per_bucket():
    torch = pytest.importorskip("torch")
    import bartels_gb300 as bg
    from bartels_gb300 import _lib
    from bartels_gb300.meshes import kuhn_cube, material_params
    ctx = bg.Context.default()
    res = []
    for n in (20, 21):  # 9,261 and 10,648 vertices: the same size bucket
        V, E = kuhn_cube(n)
        plan = bg.MeshPlan(V, E, ctx)
        plan.set_element_data(params=material_params("neohookean", len(E), 2e6, 0.45), density=np.full(len(E), 1e3))
        q = torch.from_numpy(V.ravel().copy()).cuda()
        _lib.check(bg.lib().bartels_plan_hessian_d(ctx.handle, plan.handle, 0, 1, 1e-6, 0, 1e-4, 1.0,
                                                   C.c_void_p(q.data_ptr()), None), "hessian")
        a, b = C.c_int(), C.c_int()
        _lib.check(bg.lib().bartels_plan_autotune(ctx.handle, plan.handle, None, 0, C.byref(a), C.byref(b)), "tune")
        assert a.value in (4, 8, 16) and b.value in (4, 8)
        res.append((a.value, b.value))
        plan.close()
    assert res[0] == res[1]


def test_hessian_autotuner_choice_is_cached_and_does_not_change_values():
    """Every assembly CTA shape and PSD block size gives the same Hessian bits;
    the autotuner picks one of them and a second plan of the same size bucket
    takes it from the context's cache."""
    torch = pytest.importorskip("torch")
    import bartels_gb300 as bg
    from bartels_gb300 import _lib
    from bartels_gb300.meshes import kuhn_cube, material_params
    L = bg.lib()
    ctx = bg.Context.default()
    V, E = kuhn_cube(26)
    plan = bg.MeshPlan(V, E, ctx)
    plan.set_element_data(params=material_params("neohookean", len(E), 2e6, 0.45), density=np.full(len(E), 1e3))
    rng = np.random.default_rng(4)
    q = torch.from_numpy((V * np.array([1.0, 1.0, 0.6]) + 0.01 * rng.standard_normal(V.shape)).ravel()).cuda()

    def hess():
        vals = torch.empty(plan.nnz, dtype=torch.float32, device="cuda")
        _lib.check(L.bartels_plan_hessian_d(ctx.handle, plan.handle, 0, _lib.PSD_SIMPLE_FIX, 1e-6, 0, 1e-4, 1.0,
                                            C.c_void_p(q.data_ptr()), C.c_void_p(vals.data_ptr())), "hessian")
        ctx.synchronize()
        return vals.cpu().numpy()

    ref = None
    for chunk in (128, 64):
        for block in (64, 128, 256):
            _lib.check(L.bartels_plan_set_hessian_tuning(plan.handle, chunk, block), "set tuning")
            h = hess()
            if ref is None:
                ref = h
            assert np.array_equal(h, ref), (chunk, block)
    assert L.bartels_plan_set_hessian_tuning(plan.handle, 96, 128) != 0
    c, b = C.c_int(), C.c_int()
    _lib.check(L.bartels_plan_autotune_hessian(ctx.handle, plan.handle, 0, C.c_void_p(q.data_ptr()), 1,
                                               C.byref(c), C.byref(b)), "autotune_hessian")
    assert c.value in (64, 128) and b.value in (64, 128, 256)
    assert np.array_equal(hess(), ref)
    plan.close()
    V2, E2 = kuhn_cube(28)  # 24,389 vertices against 19,683: the same bucket
    plan2 = bg.MeshPlan(V2, E2, ctx)
    plan2.set_element_data(params=material_params("neohookean", len(E2), 2e6, 0.45))
    q2 = torch.from_numpy(V2.ravel().copy()).cuda()
    c2, b2 = C.c_int(), C.c_int()
    _lib.check(L.bartels_plan_autotune_hessian(ctx.handle, plan2.handle, 0, C.c_void_p(q2.data_ptr()), 0,
                                               C.byref(c2), C.byref(b2)), "autotune_hessian")
    assert (c2.value, b2.value) == (c.value, b.value)
    plan2.close()


@pytest.mark.parametrize("precond", ["jacobi", "learned"])
def test_batched_step_matches_one_by_one(precond):
    pytest.importorskip("torch")
    import bartels_gb300 as bg
    from bartels_gb300 import batched, lpcg
    net = lpcg.LearnedPreconditioner.load(lpcg.WEIGHTS, bg.Context.default()) if precond == "learned" else None
    inst = batched.make_instances(6, seed=3, n_range=(4, 7))
    packed = batched.pack(inst)
    stats, rel, x = batched.solve(packed, tol=1e-8, precond=precond, net=net)
    assert stats["converged"] == 6 and rel.max() <= 1e-8, stats
    for k in (0, 3, 5):
        one = batched.pack([inst[k]])
        _, r1, x1 = batched.solve(one, tol=1e-8, precond=precond, net=net, autotune=False)
        assert r1.max() <= 1e-8
        xs = x[3 * packed["voff"][k]:3 * packed["voff"][k + 1]]
        assert np.linalg.norm(xs - x1) <= 1e-6 * np.linalg.norm(x1), k
    if net is not None:
        net.close()
