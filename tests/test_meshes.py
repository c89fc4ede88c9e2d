"""Mesh helpers of the workloads (bartels_gb300/meshes.py), on CPU: the Kuhn
cube's orientation and volumes, voxel carving (one connected component, no
unused vertices, cells inside the spheres), the MEDIT reader and the
per-model material parameter conventions."""
import numpy as np
import pytest
import scipy.sparse as sp
from scipy.sparse.csgraph import connected_components

from bartels_gb300.meshes import carved_cube, kuhn_cube, lame_from_young, material_params, read_medit


def signed_volumes(V, E):
    a, b, c = (V[E[:, k]] - V[E[:, 0]] for k in (1, 2, 3))
    return np.einsum("ij,ij->i", a, np.cross(b, c)) / 6.0


def test_kuhn_cube_is_positively_oriented_and_fills_the_cube():
    V, E = kuhn_cube(5, size=2.0)
    vol = signed_volumes(V, E)
    assert np.all(vol > 0) and np.allclose(vol, 8.0 / (6 * 125)) and np.isclose(vol.sum(), 8.0)


def test_carved_cube_keeps_one_component_inside_the_spheres():
    n = 12
    centers = np.array([[0.25, 0.25, 0.25], [0.8, 0.8, 0.8]])   # two disjoint balls, the first larger
    radii = np.array([0.22, 0.12])
    V, E, cent = carved_cube(n, centers, radii)
    assert E.min() == 0 and E.max() == len(V) - 1 and len(np.unique(E)) == len(V)   # every vertex used
    assert np.all(signed_volumes(V, E) > 0)
    rows = np.repeat(E, 4, axis=1).ravel()
    cols = np.tile(E, (1, 4)).ravel()
    A = sp.coo_matrix((np.ones(len(rows)), (rows, cols)), shape=(len(V), len(V)))
    assert connected_components(A, directed=False)[0] == 1
    # the kept cells are those of the larger ball
    assert np.all(np.linalg.norm(cent - centers[0], axis=1) <= radii[0] + np.sqrt(3) / n)
    assert len(E) % 6 == 0


def test_carved_cube_without_cells_is_an_error():
    with pytest.raises(ValueError):
        carved_cube(4, np.array([[5.0, 5.0, 5.0]]), np.array([0.1]))


def test_read_medit(tmp_path):
    p = tmp_path / "tet.mesh"
    p.write_text("MeshVersionFormatted 1\nDimension 3\nVertices\n4\n0 0 0 1\n1 0 0 1\n0 1 0 1\n0 0 1 1\n"
                 "Triangles\n1\n1 2 3 1\nTetrahedra\n1\n1 2 3 4 0\nEnd\n")
    V, E = read_medit(str(p))
    assert V.shape == (4, 3) and np.array_equal(E, [[0, 1, 2, 3]]) and np.isclose(signed_volumes(V, E)[0], 1 / 6)


def test_material_parameter_conventions():
    lam, mu = lame_from_young(2e6, 0.45)
    assert np.isclose(lam, 2e6 * 0.45 / (1.45 * 0.1)) and np.isclose(mu, 2e6 / 2.9)
    assert np.allclose(material_params("neohookean", 2, 2e6, 0.45), [[mu / 2, lam / 2]] * 2)
    assert np.allclose(material_params("stvk", 1, 2e6, 0.45), [[lam, mu]])
    assert np.allclose(material_params("corotational", 1, 2e6, 0.45), [[lam, mu]])
    assert np.allclose(material_params("arap", 1, 2e6, 0.45), [[lam / 2, mu]])
    assert np.allclose(material_params("linear_elasticity", 1, 2e6, 0.45), [[2e6, 0.45]])
