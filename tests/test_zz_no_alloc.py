"""bartels_tetmesh_dq_noalloc_d: the gradient entry point for callers that
cannot allocate device memory (hosts that reserve all device memory for their
own pool, loops that must not take cudaMalloc's implicit synchronisation,
hosts that account every allocation). It must give the same gradient as
bartels_tetmesh_dq, call after call, for every law, without allocating.

Kept in its own file so that pytest collects it last."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_gradient_matches_existing_entry_point():
    torch = pytest.importorskip("torch")
    import bartels_gb300 as bg
    from bartels_gb300 import _lib
    from bartels_gb300.meshes import kuhn_cube, material_params

    L = bg.lib()
    V, E = kuhn_cube(6)  # 1296 tets
    rng = np.random.default_rng(31)
    for model in bg.api.MODELS:
        params = material_params(model, len(E), 2e6, 0.45)
        plan = bg.MeshPlan(V, E)
        plan.set_element_data(params=params)
        for call in range(2):
            q = (V + rng.uniform(-0.01, 0.01, V.shape)).ravel()
            g_ref = plan.dq(model, q)  # the existing entry point
            q_d = torch.from_numpy(q).cuda()
            g_d = torch.full_like(q_d, float("nan"))
            torch.cuda.synchronize()
            free_before = torch.cuda.mem_get_info()[0]
            _lib.check(L.bartels_tetmesh_dq_noalloc_d(plan.ctx.handle, plan.handle, bg.api.MODELS[model],
                                                      C.c_void_p(q_d.data_ptr()), C.c_void_p(g_d.data_ptr())),
                       "bartels_tetmesh_dq_noalloc_d")
            plan.ctx.synchronize()
            g = g_d.cpu().numpy()
            assert np.all(np.isfinite(g))
            assert np.linalg.norm(g - g_ref) <= 1e-12 * np.linalg.norm(g_ref), (model, call)
            if call == 1:
                # the second call cannot have taken device memory
                assert torch.cuda.mem_get_info()[0] == free_before
        plan.close()


def test_noalloc_gradient_rejects_meshes_above_its_scratch():
    import bartels_gb300 as bg
    from bartels_gb300 import _lib
    from bartels_gb300.meshes import kuhn_cube
    torch = pytest.importorskip("torch")

    V, E = kuhn_cube(23)  # 73,002 tets > 65,536
    plan = bg.MeshPlan(V, E)
    q_d = torch.zeros(3 * len(V), dtype=torch.float64, device="cuda")
    g_d = torch.zeros_like(q_d)
    s = bg.lib().bartels_tetmesh_dq_noalloc_d(plan.ctx.handle, plan.handle, _lib.NEOHOOKEAN,
                                              C.c_void_p(q_d.data_ptr()), C.c_void_p(g_d.data_ptr()))
    assert s == _lib.E_UNSUPPORTED
    assert b"65536" in bg.lib().bartels_last_error()
    plan.close()
