"""Regenerate the golden fixtures in this folder from the reference's data files.

Reads (read-only) the Bartels source tree given as the one required argument
and writes compressed .npz fixtures:

* coarser_bunny.npz   V (500,3), E (1518,4) 0-based  <- data/meshes_mesh/coarser_bunny.mesh
* tet.npz, two_tets.npz                               <- data/meshes_mesh/{tet,two_tets}.mesh
* cube6.npz           6-tet cube                      <- data/meshes_tetgen/Cube/cube.{node,ele}
* H_neohookean_coarser_bunny.npz  CSR of data/matrices/H_neohookean_coarser_bunny.txt
* M_coarse_bunny.npz              CSR of data/matrices/M_coarse_bunny.txt
* M_two_tets.npz                  CSR of data/matrices/M_two_tets.txt

MatrixMarket entries are kept exactly as stored (explicit zeros included), so
the CSR pattern of each fixture is the reference's assembled pattern.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def read_medit(path):
    """Minimal MEDIT .mesh reader: Vertices + Tetrahedra (1-based) sections."""
    toks = open(path).read().split()
    V = E = None
    i = 0
    while i < len(toks):
        t = toks[i]
        if t == "Vertices":
            n = int(toks[i + 1])
            vals = np.array(toks[i + 2:i + 2 + 4 * n], dtype=np.float64).reshape(n, 4)
            V = vals[:, :3].copy()
            i += 2 + 4 * n
        elif t == "Tetrahedra":
            n = int(toks[i + 1])
            vals = np.array(toks[i + 2:i + 2 + 5 * n], dtype=np.int64).reshape(n, 5)
            E = (vals[:, :4] - 1).astype(np.int32)
            i += 2 + 5 * n
        else:
            i += 1
    return V, E


def read_tetgen(node, ele):
    nl = [l.split() for l in open(node) if l.strip() and not l.lstrip().startswith("#")]
    n = int(nl[0][0])
    V = np.array([[float(x) for x in r[1:4]] for r in nl[1:1 + n]])
    el = [l.split() for l in open(ele) if l.strip() and not l.lstrip().startswith("#")]
    m = int(el[0][0])
    E = np.array([[int(x) for x in r[1:5]] for r in el[1:1 + m]], dtype=np.int32)
    return V, E


def read_mm(path):
    with open(path) as f:
        header = f.readline()
        assert "coordinate" in header and "real" in header
        line = f.readline()
        while line.startswith("%"):
            line = f.readline()
        nr, nc, nnz = (int(x) for x in line.split())
        data = np.loadtxt(f, dtype=np.float64, max_rows=nnz, ndmin=2)
    r = data[:, 0].astype(np.int64) - 1
    c = data[:, 1].astype(np.int64) - 1
    v = data[:, 2]
    order = np.lexsort((c, r))
    r, c, v = r[order], c[order], v[order]
    assert not np.any((np.diff(r) == 0) & (np.diff(c) == 0)), "duplicate entries"
    row_ptr = np.zeros(nr + 1, np.int64)
    np.add.at(row_ptr, r + 1, 1)
    row_ptr = np.cumsum(row_ptr).astype(np.int32)
    return dict(shape=np.array([nr, nc]), row_ptr=row_ptr, col=c.astype(np.int32), val=v)


def main(ref):
    d = os.path.join(ref, "data")
    V, E = read_medit(os.path.join(d, "meshes_mesh", "coarser_bunny.mesh"))
    np.savez_compressed(os.path.join(HERE, "coarser_bunny.npz"), V=V, E=E)
    for name in ("tet", "two_tets"):
        V, E = read_medit(os.path.join(d, "meshes_mesh", name + ".mesh"))
        np.savez_compressed(os.path.join(HERE, name + ".npz"), V=V, E=E)
    V, E = read_tetgen(os.path.join(d, "meshes_tetgen", "Cube", "cube.node"),
                       os.path.join(d, "meshes_tetgen", "Cube", "cube.ele"))
    np.savez_compressed(os.path.join(HERE, "cube6.npz"), V=V, E=E)
    for src, dst in (("H_neohookean_coarser_bunny.txt", "H_neohookean_coarser_bunny.npz"),
                     ("M_coarse_bunny.txt", "M_coarse_bunny.npz"),
                     ("M_two_tets.txt", "M_two_tets.npz")):
        m = read_mm(os.path.join(d, "matrices", src))
        np.savez_compressed(os.path.join(HERE, dst), **m)
        print(dst, m["shape"], len(m["val"]))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the Bartels source tree>")
    main(sys.argv[1])
