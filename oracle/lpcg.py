"""NumPy restatement of the learned preconditioner's network, loss and gradient.

TEST INFRASTRUCTURE ONLY: the checker of the GPU forward / backward kernels
(bartels_gb300/csrc/lpcg.cu, gemm_tc.cu). The reference has no learned
preconditioner (its linear solver is Eigen::SparseLU,
include/search_direction_newton_sparse.h:8), so this module restates the
library's own published design, not a reference routine:

  Ahat = L^-1 A L^-T (L_v = chol(A_vv)), network over the block pattern,
  Ghat = network output (block-lower-triangular), G = Ghat L^-1, M^-1 = G^T G,
  loss = log(tr(Ghat Ahat Ghat^T) / N) - (2/N) sum log diag(Ghat)   (Kaporin),
  trace estimated with probes w: tr ~ (1/P) sum_p (Ghat^T w)^T Ahat (Ghat^T w).

With ``bf16=True`` the tensor-core GEMM inputs (activations and weights) are
rounded to BF16 exactly where the GPU rounds them; with ``bf16=False`` the
whole computation is plain float64 (used for finite-difference checks of the
backward formulas).
"""
from __future__ import annotations

import numpy as np

H, LAYERS, DX, DE = 64, 3, 4, 10


def layout():
    """name -> (offset, shape) of the flat FP32 parameter vector."""
    out, o = {}, 0

    def take(name, shape):
        nonlocal o
        out[name] = (o, shape)
        o += int(np.prod(shape))

    take("W0", (DX, H))
    take("b0", (H,))
    for l in range(LAYERS):
        take(f"Wpq{l}", (2 * H, H))   # out x in
        take(f"We{l}", (DE, H))
        take(f"be{l}", (H,))
        take(f"Wu{l}", (H, 2 * H))    # out x in
        take(f"bu{l}", (H,))
    take("Wst", (2 * H, H))
    take("Wf", (DE, H))
    take("bf", (H,))
    take("Wo", (H, 9))
    take("bo", (9,))
    take("Wd", (H, 6))
    take("bd", (6,))
    take("Wskip", (DE, 9))
    return out, o


LAYOUT, NPARAMS = layout()


def unpack(theta):
    return {k: theta[o:o + int(np.prod(s))].reshape(s).astype(np.float64) for k, (o, s) in LAYOUT.items()}


def pack(d):
    theta = np.zeros(NPARAMS)
    for k, (o, s) in LAYOUT.items():
        theta[o:o + int(np.prod(s))] = np.asarray(d[k]).ravel()
    return theta


def bf16(x):
    """Round to BF16 (nearest even) and return as float64."""
    f = np.ascontiguousarray(np.asarray(x, np.float64).astype(np.float32))
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u >> 16) & 1) + 0x7FFF
    u2 = ((u + r) & 0xFFFF0000).astype(np.uint32)
    return u2.view(np.float32).astype(np.float64)


def rademacher(seed, nprobe, n):
    """The GPU's probe vectors: hash3(seed, p, i) & 1 -> +1 / -1."""
    M = np.uint64(0xFFFFFFFF)
    a = np.uint64(seed)
    i = np.arange(n, dtype=np.uint64)
    out = np.empty((nprobe, n))
    for p in range(nprobe):
        h = ((a * np.uint64(0x9E3779B1)) & M) ^ (((np.uint64(p) + np.uint64(0x7F4A7C15)) * np.uint64(0x85EBCA77)) & M) \
            ^ (((i + np.uint64(0x165667B1)) * np.uint64(0xC2B2AE3D)) & M)
        h = h & M
        h ^= h >> np.uint64(15)
        h = (h * np.uint64(0x2C1B3C6D)) & M
        h ^= h >> np.uint64(12)
        h = (h * np.uint64(0x297A2D39)) & M
        h ^= h >> np.uint64(15)
        out[p] = np.where(h & np.uint64(1), 1.0, -1.0)
    return out


class Graph:
    """Block pattern of a plan (sorted rows, self included) and its maps."""

    def __init__(self, brp, bcol, pinned):
        self.brp = np.asarray(brp, np.int64)
        self.bcol = np.asarray(bcol, np.int64)
        self.nV = len(self.brp) - 1
        self.row = np.repeat(np.arange(self.nV), np.diff(self.brp))
        self.pinned = np.zeros(self.nV, bool) if pinned is None else np.asarray(pinned, bool)
        self.diag = np.array([np.searchsorted(self.bcol[self.brp[v]:self.brp[v + 1]], v) for v in range(self.nV)])
        pos = {(int(self.row[p]), int(self.bcol[p])): p for p in range(len(self.bcol))}
        self.rev = np.array([pos[(int(self.bcol[p]), int(self.row[p]))] for p in range(len(self.bcol))])
        free_edge = ~self.pinned[self.row] & ~self.pinned[self.bcol]
        self.edge = free_edge & (self.row != self.bcol)           # directed message edges
        self.lower = free_edge & (self.bcol < self.row)            # off-diagonal lower blocks
        self.dpos = self.brp[:-1] + self.diag                      # diagonal positions


def blocks_from_csr(brp, bcol, values):
    """[nnzb, 3, 3] blocks from values in the plan's scalar-CSR order."""
    brp = np.asarray(brp)
    nV = len(brp) - 1
    out = np.empty((brp[-1], 3, 3))
    for v in range(nV):
        nb = brp[v + 1] - brp[v]
        seg = np.asarray(values[9 * brp[v]:9 * brp[v + 1]], np.float64).reshape(3, nb, 3)
        out[brp[v]:brp[v + 1]] = seg.transpose(1, 0, 2)
    return out


def features(g, A):
    """Linv (nV,3,3), Ahat (nnzb,3,3) with zeros on pinned blocks, x (nV,4), invdeg."""
    D = A[g.dpos]
    L = np.linalg.cholesky(D)
    Li = np.linalg.inv(L)
    Li[g.pinned] = np.eye(3)
    Ah = np.einsum("pkm,pml,pnl->pkn", Li[g.row], A, Li[g.bcol])
    blocked = g.pinned[g.row] | g.pinned[g.bcol]
    Ah[blocked] = 0.0
    nrm = np.sqrt((Ah ** 2).sum(axis=(1, 2)))
    fe = np.concatenate([Ah.reshape(-1, 9), nrm[:, None]], axis=1)
    deg = np.bincount(g.row[g.edge], minlength=g.nV).astype(np.float64)
    s = np.bincount(g.row[g.edge], weights=nrm[g.edge], minlength=g.nV)
    mx = np.zeros(g.nV)
    np.maximum.at(mx, g.row[g.edge], nrm[g.edge])
    x = np.stack([np.ones(g.nV), deg / 14.0, np.where(deg > 0, s / np.maximum(deg, 1), 0.0), mx], axis=1)
    x[g.pinned] = 0.0
    invdeg = np.where(deg > 0, 1.0 / np.maximum(deg, 1), 0.0)
    invdeg[g.pinned] = 0.0
    return Li, Ah, fe, x, invdeg


def forward(g, A, theta, bf=True):
    """Network outputs: raw Ghat blocks per lower position (dict) and cache."""
    P = unpack(theta)
    rnd = bf16 if bf else (lambda t: np.asarray(t, np.float64))
    Li, Ah, fe, x, invdeg = features(g, A)
    c = dict(Li=Li, Ah=Ah, fe=fe, x=x, invdeg=invdeg)
    pre0 = x @ P["W0"] + P["b0"]
    h = np.maximum(pre0, 0.0)
    c["pre0"] = pre0
    c["h"], c["ha"], c["pq"], c["upre"] = [h], [], [], []
    e = g.edge
    for l in range(LAYERS):
        hb = rnd(h)
        pq = hb @ rnd(P[f"Wpq{l}"]).T
        Pm, Q = pq[:, :H], pq[:, H:]
        r = fe @ P[f"We{l}"] + P[f"be{l}"]
        m = np.maximum(Pm[g.row] + Q[g.bcol] + r, 0.0) * e[:, None]
        a = np.zeros((g.nV, H))
        np.add.at(a, g.row, m)
        a *= invdeg[:, None]
        ha = np.concatenate([hb, rnd(a)], axis=1)
        u = ha @ rnd(P[f"Wu{l}"]).T + P[f"bu{l}"]
        c["ha"].append(ha)
        c["pq"].append(pq)
        c["upre"].append(u)
        h = h + np.maximum(u, 0.0)
        c["h"].append(h)
    hb = rnd(h)
    c["hb3"] = hb
    st = hb @ rnd(P["Wst"]).T
    c["st"] = st
    S, T = st[:, :H], st[:, H:]
    lo = g.lower
    zpre = S[g.row] + T[g.bcol] + fe @ P["Wf"] + P["bf"]
    z = np.maximum(zpre, 0.0) * lo[:, None]
    Gh = (z @ P["Wo"] + P["bo"] + fe @ P["Wskip"]) * lo[:, None]
    d = h @ P["Wd"] + P["bd"]
    d[g.pinned] = 0.0
    c.update(zpre=zpre, z=z, Gh=Gh, d=d)
    return c


def ghat_blocks(g, c):
    """Ghat as 3x3 blocks at every pattern position (zero above the diagonal)."""
    Gb = np.zeros((len(g.bcol), 3, 3))
    Gb[g.lower] = c["Gh"][g.lower].reshape(-1, 3, 3)
    d = c["d"]
    Dg = np.zeros((g.nV, 3, 3))
    Dg[:, 0, 0], Dg[:, 1, 1], Dg[:, 2, 2] = np.exp(d[:, 0]), np.exp(d[:, 1]), np.exp(d[:, 2])
    Dg[:, 1, 0], Dg[:, 2, 0], Dg[:, 2, 1] = d[:, 3], d[:, 4], d[:, 5]
    Dg[g.pinned] = 0.0
    Gb[g.dpos] = Dg
    return Gb


def factor_blocks(g, c):
    """G = Ghat L^-1 per pattern block (lower part; zero for pinned)."""
    Gb = ghat_blocks(g, c)
    return np.einsum("pkm,pml->pkl", Gb, c["Li"][g.bcol])


def loss_and_grad(g, A, theta, probes, bf=True):
    """Loss and d loss / d theta for the given probe vectors (P, 3nV)."""
    Pm = unpack(theta)
    c = forward(g, A, theta, bf)
    rnd = bf16 if bf else (lambda t: np.asarray(t, np.float64))
    W = np.asarray(probes, np.float64).reshape(len(probes), g.nV, 3)
    W[:, g.pinned] = 0.0
    Gb = ghat_blocks(g, c)
    Gb[g.pinned[g.row] | g.pinned[g.bcol]] = 0.0
    npr = W.shape[0]
    # u_p[j] = sum_i Ghat_ij^T w_p[i]
    U = np.zeros_like(W)
    contrib = np.einsum("pkl,qpk->qpl", Gb, W[:, g.row])
    for q in range(npr):
        np.add.at(U[q], g.bcol, contrib[q])
    # v = Ahat u
    V = np.zeros_like(W)
    cv = np.einsum("pkl,qpl->qpk", c["Ah"], U[:, g.bcol])
    for q in range(npr):
        np.add.at(V[q], g.row, cv[q])
    V[:, g.pinned] = 0.0
    t = float((U * V).sum()) / npr
    free = ~g.pinned
    nf = 3.0 * free.sum()
    ld = float(c["d"][free, :3].sum())
    loss = np.log(t / nf) - 2.0 * ld / nf
    ct, cl = 2.0 / (npr * t), 2.0 / nf
    # d Ghat_ij = ct sum_p w_p[i] (x) v_p[j]
    dGb = ct * np.einsum("qpk,qpl->pkl", W[:, g.row], V[:, g.bcol])
    dG = np.zeros((len(g.bcol), 9))
    dG[g.lower] = dGb[g.lower].reshape(-1, 9)
    dd = np.zeros((g.nV, 6))
    Dd = dGb[g.dpos]
    dd[:, 0] = Dd[:, 0, 0] * np.exp(c["d"][:, 0]) - cl
    dd[:, 1] = Dd[:, 1, 1] * np.exp(c["d"][:, 1]) - cl
    dd[:, 2] = Dd[:, 2, 2] * np.exp(c["d"][:, 2]) - cl
    dd[:, 3], dd[:, 4], dd[:, 5] = Dd[:, 1, 0], Dd[:, 2, 0], Dd[:, 2, 1]
    dd[g.pinned] = 0.0
    grad = {}
    # head
    lo = g.lower
    dz = (dG @ Pm["Wo"].T) * lo[:, None]
    dzpre = dz * (c["zpre"] > 0)
    grad["Wo"] = c["z"].T @ dG
    grad["bo"] = dG.sum(0)
    grad["Wf"] = c["fe"].T @ dzpre
    grad["bf"] = dzpre.sum(0)
    grad["Wskip"] = (c["fe"] * lo[:, None]).T @ dG
    grad["Wd"] = c["h"][-1].T @ dd
    grad["bd"] = dd.sum(0)
    dS = np.zeros((g.nV, H))
    dT = np.zeros((g.nV, H))
    np.add.at(dS, g.row, dzpre)
    np.add.at(dT, g.bcol, dzpre)
    dst = np.concatenate([dS, dT], axis=1)
    grad["Wst"] = dst.T @ c["hb3"]
    dh = dd @ Pm["Wd"].T + rnd(dst) @ rnd(Pm["Wst"])
    e = g.edge
    for l in reversed(range(LAYERS)):
        du = dh * (c["upre"][l] > 0)
        grad[f"Wu{l}"] = du.T @ c["ha"][l]
        grad[f"bu{l}"] = du.sum(0)
        dha = rnd(du) @ rnd(Pm[f"Wu{l}"])
        dh = dh + dha[:, :H]
        da = dha[:, H:] * c["invdeg"][:, None]
        pq = c["pq"][l]
        pre = pq[g.row, :H] + pq[g.bcol, H:] + c["fe"] @ Pm[f"We{l}"] + Pm[f"be{l}"]
        dpre = da[g.row] * (pre > 0) * e[:, None]
        grad[f"We{l}"] = c["fe"].T @ dpre
        grad[f"be{l}"] = dpre.sum(0)
        dP = np.zeros((g.nV, H))
        dQ = np.zeros((g.nV, H))
        np.add.at(dP, g.row, dpre)
        np.add.at(dQ, g.bcol, dpre)
        dpq = np.concatenate([dP, dQ], axis=1)
        grad[f"Wpq{l}"] = dpq.T @ c["ha"][l][:, :H]
        dh = dh + rnd(dpq) @ rnd(Pm[f"Wpq{l}"])
    dpre0 = dh * (c["pre0"] > 0)
    grad["W0"] = c["x"].T @ dpre0
    grad["b0"] = dpre0.sum(0)
    return loss, pack(grad), t


def factor_pcg_iterations(Hs, G, b, tol=1e-8, maxit=20000):
    """Iterations of PCG on sparse Hs with M^-1 = G^T G (dense or sparse G)."""
    x = np.zeros_like(b)
    r = b.copy()
    z = G.T @ (G @ r)
    p = z.copy()
    rz = r @ z
    b2 = b @ b
    for it in range(maxit):
        q = Hs @ p
        a = rz / (p @ q)
        x += a * p
        r -= a * q
        if r @ r <= tol * tol * b2:
            return it + 1
        z = G.T @ (G @ r)
        rz2 = r @ z
        p = z + (rz2 / rz) * p
        rz = rz2
    return maxit
