"""The heterogeneous stress case (carved cube, log-normal stiffness with 100x
inclusions, axial compression) on a small grid: both preconditioners reach
the Newton tolerance in every load step, the learned one with block-Jacobi as
its fallback, and the final state's energy and gradient match the FP64 CPU
restatement."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_stress_case_small(oracle):
    pytest.importorskip("torch")
    import bartels_gb300 as bg
    from bartels_gb300 import lpcg, stress_case
    prob = stress_case.build(n=16, seed=1)
    assert prob["bottom"].any() and prob["top"].any()
    net = lpcg.LearnedPreconditioner.load(lpcg.WEIGHTS, bg.Context.default())
    res = {}
    for pc in ("jacobi", "learned"):
        rows, tot, q = stress_case.run(prob, pc, net, steps=3, compression=0.15, gradient_tol=1e-5, max_newton=40,
                                       log=lambda s: None)
        assert all(r["converged"] for r in rows), rows
        # the final state's FP64 energy and gradient against the restatement
        V, E, params, qf = prob["V"], prob["E"], prob["params"], q.ravel()
        dphi, vol = oracle.dphi_dX(V, E), oracle.volume(V, E)
        plan = bg.MeshPlan(V, E)
        e, g = plan.q("neohookean", qf, dphi, vol, params), plan.dq("neohookean", qf, dphi, vol, params)
        e_ref = oracle.tetmesh_q("neohookean", E, qf, dphi, vol, params)
        g_ref = oracle.tetmesh_dq("neohookean", len(V), E, qf, dphi, vol, params)
        assert abs(e - e_ref) < 1e-10 * abs(e_ref) and abs(tot["energy"] - e_ref) < 1e-10 * abs(e_ref)
        assert np.linalg.norm(g - g_ref) < 1e-9 * np.linalg.norm(g_ref)
        plan.close()
        res[pc] = (tot, q)
    # same equilibrium from both solvers
    qa, qb = res["jacobi"][1], res["learned"][1]
    assert np.linalg.norm(qa - qb) <= 1e-4 * np.linalg.norm(qa)
    # the learned factor needs fewer PCG iterations than block-Jacobi on this unseen material
    assert res["learned"][0]["pcg_per_newton"] < res["jacobi"][0]["pcg_per_newton"]
    net.close()
