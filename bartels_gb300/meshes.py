"""Mesh helpers: the Kuhn-subdivided cube used by the benchmarks and a MEDIT reader.

Kuhn cube: (n+1)^3 grid vertices on [0, size]^3, vertex id i + (n+1)(j + (n+1)k);
every cell is split into the 6 tets that share its (0,0,0)-(1,1,1) diagonal, so
face diagonals agree between neighbouring cells (a conforming mesh). Tets are
numbered cell-major (6 consecutive tets per cell) and positively oriented.
"""
from __future__ import annotations

import itertools

import numpy as np


def kuhn_cube(n: int, size: float = 1.0):
    """Return V (nV, 3) float64 and E (nT, 4) int32 for an n^3-cell Kuhn cube."""
    if n < 1:
        raise ValueError("n must be >= 1")
    m = n + 1
    g = np.arange(m, dtype=np.float64) * (size / n)
    k, j, i = np.meshgrid(np.arange(m), np.arange(m), np.arange(m), indexing="ij")
    V = np.stack([g[i.ravel()], g[j.ravel()], g[k.ravel()]], axis=1)
    ci, cj, ck = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    # cell-major order with x fastest: cell = i + n (j + n k)
    ci, cj, ck = ck.ravel(), cj.ravel(), ci.ravel()
    base = ci + m * (cj + m * ck)
    step = np.array([1, m, m * m])
    tets = []
    for perm in itertools.permutations(range(3)):
        p0 = base
        p1 = p0 + step[perm[0]]
        p2 = p1 + step[perm[1]]
        p3 = p2 + step[perm[2]]
        sign = np.linalg.det(np.eye(3)[list(perm)])
        tets.append(np.stack([p0, p1, p2, p3] if sign > 0 else [p0, p2, p1, p3], axis=1))
    E = np.stack(tets, axis=1).reshape(-1, 4).astype(np.int32)
    return V, E


def cube_counts(n: int):
    """Vertex, tet, edge and Hessian-nnz counts of kuhn_cube(n)."""
    nv = (n + 1) ** 3
    nt = 6 * n ** 3
    edges = 3 * n * (n + 1) ** 2 + 3 * n ** 2 * (n + 1) + n ** 3
    return dict(nV=nv, nT=nt, edges=edges, nnz=9 * (nv + 2 * edges), ndof=3 * nv)


def read_medit(path: str):
    """Vertices and (1-based) Tetrahedra of a MEDIT .mesh file -> V, E (0-based)."""
    toks = open(path).read().split()
    V = E = None
    i = 0
    while i < len(toks):
        t = toks[i]
        if t == "Vertices":
            n = int(toks[i + 1])
            V = np.array(toks[i + 2:i + 2 + 4 * n], dtype=np.float64).reshape(n, 4)[:, :3].copy()
            i += 2 + 4 * n
        elif t == "Tetrahedra":
            n = int(toks[i + 1])
            E = (np.array(toks[i + 2:i + 2 + 5 * n], dtype=np.int64).reshape(n, 5)[:, :4] - 1).astype(np.int32)
            i += 2 + 5 * n
        else:
            i += 1
    return V, E


def lame_from_young(E, nu):
    """(lambda, mu) from Young's modulus and Poisson ratio (matlab/emu_to_lame.m:17-18)."""
    lam = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu))
    mu = E / (2.0 * (1.0 + nu))
    return lam, mu


def material_params(model: str, nT: int, young: float, nu: float):
    """Per-tet params in the reference's convention: Neo-Hookean (mu/2, lambda/2)
    (the reference's README.md:50, matlab/examples/test_tet_materials.m:64), StVK and corotational (lambda, mu),
    ARAP (lambda/2, mu) with k = lambda/2 in column 0 (matlab/examples/test_tet_materials.m:80),
    linear elasticity (Young's modulus, Poisson ratio) (src/d2psi_linear_elasticity_de2.cpp:10-11)."""
    lam, mu = lame_from_young(young, nu)
    if model.startswith("neohookean"):
        row = (0.5 * mu, 0.5 * lam)
    elif model == "arap":
        row = (0.5 * lam, mu)
    elif model == "linear_elasticity":
        row = (young, nu)
    else:
        row = (lam, mu)
    return np.tile(np.array(row, dtype=np.float64), (nT, 1))


def carved_cube(n: int, centers, radii, size: float = 1.0):
    """Voxel carving of the n^3 Kuhn cube: keep the cells whose centre lies in
    the union of the spheres (centers (k, 3), radii (k,)), then the largest
    vertex-connected component. Returns V, E (renumbered) and the kept cell
    centres per tet (for per-tet material fields)."""
    V, E = kuhn_cube(n, size)
    centers = np.asarray(centers, dtype=np.float64)
    radii = np.asarray(radii, dtype=np.float64)
    c = V[E].mean(axis=1)  # tet centroids
    cell = np.arange(len(E)) // 6
    m = n
    ci = cell % m
    cj = (cell // m) % m
    ck = cell // (m * m)
    cc = (np.stack([ci, cj, ck], axis=1) + 0.5) * (size / n)
    d2 = ((cc[:, None, :] - centers[None, :, :]) ** 2).sum(axis=2)
    keep = (d2 <= radii[None, :] ** 2).any(axis=1)
    E = E[keep]
    c = c[keep]
    # largest connected component (union-find over tet vertices)
    parent = np.arange(len(V))

    def find(a):
        root = a
        while parent[root] != root:
            root = parent[root]
        while parent[a] != root:
            parent[a], a = root, parent[a]
        return root

    for t in E:
        r0 = find(t[0])
        for k in range(1, 4):
            rk = find(t[k])
            if rk != r0:
                parent[rk] = r0
    roots = np.array([find(v) for v in E[:, 0]])
    if len(roots) == 0:
        raise ValueError("no cell inside the spheres")
    vals, counts = np.unique(roots, return_counts=True)
    big = vals[np.argmax(counts)]
    E = E[roots == big]
    c = c[roots == big]
    used = np.unique(E.ravel())
    remap = -np.ones(len(V), dtype=np.int64)
    remap[used] = np.arange(len(used))
    return V[used].copy(), remap[E].astype(np.int32), c
