"""The learned preconditioner's CPU restatement (oracle/lpcg.py): its hand-written
backward against finite differences, its block-Jacobi starting point, and the
parameter layout shared with the library's Python side."""
import numpy as np
import pytest

from oracle import lpcg as L


def small_system(n=3, seed=0, pin=True):
    from oracle import oracle as O
    from bartels_gb300.meshes import kuhn_cube, material_params
    V, E = kuhn_cube(n)
    rng = np.random.default_rng(seed)
    params = material_params("neohookean", len(E), 2e6, 0.45)
    dphi, vol = O.dphi_dX(V, E), O.volume(V, E)
    q = (V + 0.02 / n * rng.uniform(-1, 1, V.shape)).ravel()
    K = O.tetmesh_dq2("neohookean", len(V), E, q, dphi, vol, params, psd_tol=1e-6)
    M = O.mass_matrix(len(V), E, np.full(len(E), 1000.0), vol)
    Hs = (M + 1e-3 * K).tocsr()
    Hs.sort_indices()
    # block pattern from the scalar CSR (rows 3v carry the block columns)
    rp, ci = Hs.indptr, Hs.indices
    brp = [0]
    bcol = []
    for v in range(len(V)):
        cols = ci[rp[3 * v]:rp[3 * v + 1]][::3] // 3
        bcol += list(cols)
        brp.append(len(bcol))
    brp, bcol = np.array(brp), np.array(bcol)
    A = np.zeros((len(bcol), 3, 3))
    for v in range(len(V)):
        for b in range(brp[v], brp[v + 1]):
            j = bcol[b]
            A[b] = Hs[3 * v:3 * v + 3, 3 * j:3 * j + 3].toarray()
    pinned = (np.abs(V[:, 2]) < 1e-12) if pin else np.zeros(len(V), bool)
    return L.Graph(brp, bcol, pinned), A, Hs, pinned


def random_theta(seed, head_scale=0.05):
    from bartels_gb300.lpcg import init_params
    th = init_params(seed).astype(np.float64)
    rng = np.random.default_rng(seed + 100)
    for k in ("Wo", "bo", "Wd", "bd"):
        o, s = L.LAYOUT[k]
        th[o:o + int(np.prod(s))] = head_scale * rng.standard_normal(int(np.prod(s)))
    for l in range(L.LAYERS):
        for k in (f"be{l}", f"bu{l}"):
            o, s = L.LAYOUT[k]
            th[o:o + int(np.prod(s))] = 0.1 * rng.standard_normal(int(np.prod(s)))
    return th


def test_layout_matches_package():
    from bartels_gb300 import lpcg as P
    assert P.NPARAMS == L.NPARAMS
    assert P.LAYOUT == L.LAYOUT


def test_backward_matches_finite_differences():
    g, A, _, _ = small_system(3)
    th = random_theta(1)
    probes = L.rademacher(7, 3, 3 * g.nV)
    loss, grad, _ = L.loss_and_grad(g, A, th, probes, bf=False)
    rng = np.random.default_rng(3)
    eps = 1e-6
    for k in range(6):
        d = rng.standard_normal(L.NPARAMS)
        d /= np.linalg.norm(d)
        lp = L.loss_and_grad(g, A, th + eps * d, probes, bf=False)[0]
        lm = L.loss_and_grad(g, A, th - eps * d, probes, bf=False)[0]
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - grad @ d) <= 1e-5 * max(1.0, abs(fd)), (k, fd, grad @ d)
    # a few single coordinates in each parameter group
    for name in ("W0", "Wpq0", "We1", "Wu2", "Wst", "Wf", "Wo", "bd"):
        o, s = L.LAYOUT[name]
        i = o + int(np.prod(s)) // 3
        e = np.zeros(L.NPARAMS)
        e[i] = 1.0
        fd = (L.loss_and_grad(g, A, th + eps * e, probes, bf=False)[0]
              - L.loss_and_grad(g, A, th - eps * e, probes, bf=False)[0]) / (2 * eps)
        assert abs(fd - grad[i]) <= 1e-5 * max(1.0, abs(fd)), (name, fd, grad[i])


def test_zero_head_is_block_jacobi():
    g, A, Hs, pinned = small_system(3)
    from bartels_gb300.lpcg import init_params
    c = L.forward(g, A, init_params(0).astype(np.float64))
    G = L.factor_blocks(g, c)
    # G^T G restricted to the diagonal blocks of free vertices = D^-1, zero elsewhere
    free = np.nonzero(~pinned)[0]
    for v in free[:20]:
        Gv = G[g.dpos[v]]
        assert np.allclose(Gv.T @ Gv, np.linalg.inv(A[g.dpos[v]]), rtol=1e-9, atol=0)
    off = G[g.lower]
    assert np.all(off == 0.0)


def test_loss_of_block_jacobi_is_log_kaporin():
    """At the block-Jacobi start, the exact trace is N (Ahat has unit diagonal), so
    with many probes the loss tends to log(1) - 0 = 0."""
    g, A, _, _ = small_system(3)
    from bartels_gb300.lpcg import init_params
    th = init_params(0).astype(np.float64)
    probes = L.rademacher(11, 64, 3 * g.nV)
    loss, grad, t = L.loss_and_grad(g, A, th, probes, bf=False)
    nf = 3 * (~g.pinned).sum()
    assert abs(t / nf - 1.0) < 0.05
    assert abs(loss) < 0.05


def _factor_matrix(g, G):
    """Sparse 3nV x 3nV G from its pattern blocks (lower part incl. the diagonal)."""
    import scipy.sparse as sp
    rows, cols, vals = [], [], []
    for p in np.nonzero(g.lower | (g.row == g.bcol))[0]:
        v, j = g.row[p], g.bcol[p]
        for k in range(3):
            for l in range(3):
                rows.append(3 * v + k)
                cols.append(3 * j + l)
                vals.append(G[p, k, l])
    n = 3 * g.nV
    return sp.csr_matrix((vals, (rows, cols)), shape=(n, n))


def test_shipped_weights_beat_block_jacobi_on_an_unseen_system():
    """The shipped network (bartels_gb300/weights), evaluated by the restatement
    with the GPU's BF16 rounding on a cube it was not trained on, gives a factor
    with a positive diagonal and fewer PCG iterations than block-Jacobi."""
    from bartels_gb300 import lpcg
    g, A, Hs, pinned = small_system(8, seed=3)
    theta = np.load(lpcg.WEIGHTS)["params"].astype(np.float64)
    assert theta.shape == (sum(int(np.prod(s)) for _, s in L.LAYOUT.values()),) and np.all(np.isfinite(theta))
    free = np.repeat(~pinned, 3)
    Hf = Hs[free][:, free]
    b = np.random.default_rng(5).standard_normal(int(free.sum()))
    its = {}
    for name, th in (("learned", theta), ("block_jacobi", lpcg.init_params(0).astype(np.float64))):
        c = L.forward(g, A, th, bf=True)
        Gb = L.factor_blocks(g, c)
        d = np.array([np.diag(Gb[g.dpos[v]]) for v in np.nonzero(~pinned)[0]])
        assert np.all(d > 0)
        Gm = _factor_matrix(g, Gb)[free][:, free]
        its[name] = L.factor_pcg_iterations(Hf, Gm, b)
    assert its["learned"] < 0.9 * its["block_jacobi"], its
