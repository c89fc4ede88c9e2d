"""GB300 (sm_103a) implementation of the tet-mesh hyperelastic path of Bartels
(and its planar triangle-mesh family).

The compute lives in libbartels_gpu.so (C ABI: include/bartels_gpu.h); this
package mirrors the reference's mesh-level functions on top of it.
"""
from ._lib import (BartelsError, CONVERGED, MAX_ITERATIONS_REACHED, NEOHOOKEAN, STVK, COROTATIONAL,
                   NEOHOOKEAN_ISOCHORIC, ARAP, LINEAR_ELASTICITY, PSD_NONE, PSD_SIMPLE_FIX, LIB_PATH, lib)
from .api import (Context, MeshPlan, newton_params, linear_tetmesh_dphi_dX, volume,
                  linear_tetmesh_neohookean_q, linear_tetmesh_neohookean_dq, linear_tetmesh_neohookean_dq2,
                  linear_tetmesh_stvk_q, linear_tetmesh_stvk_dq, linear_tetmesh_stvk_dq2,
                  linear_tetmesh_corotational_q, linear_tetmesh_corotational_dq, linear_tetmesh_corotational_dq2,
                  linear_tetmesh_arap_q, linear_tetmesh_arap_dq, linear_tetmesh_arap_dq2,
                  linear_tetmesh_linear_elasticity_q, linear_tetmesh_linear_elasticity_dq,
                  linear_tetmesh_linear_elasticity_dq2,
                  linear_tetmesh_mass_matrix, linear_tetmesh_const_ext_force, fixed_point_constraint_matrix,
                  find_min_vertices, search_direction_newton_sparse, linesearch_backtracking_bisection,
                  Tri2DPlan, linear_tri2dmesh_dphi_dX, triangle_areas,
                  linear_tri2dmesh_neohookean_q, linear_tri2dmesh_neohookean_dq, linear_tri2dmesh_neohookean_dq2,
                  linear_tri2dmesh_stvk_q, linear_tri2dmesh_stvk_dq, linear_tri2dmesh_stvk_dq2,
                  linear_tri2dmesh_corotational_q, linear_tri2dmesh_corotational_dq,
                  linear_tri2dmesh_corotational_dq2, linear_tri2dmesh_arap_q, linear_tri2dmesh_arap_dq,
                  linear_tri2dmesh_arap_dq2, linear_tri2dmesh_linear_elasticity_dq2, linear_tri2dmesh_mass_matrix,
                  Tri3DPlan, linear_tri3dmesh_dphi_dX, triangle_areas_3d, triangle_normals,
                  linear_tri3dmesh_stvk_dq2, pointwise_laws, psi_neohookean_F, dpsi_neohookean_dF,
                  d2psi_neohookean_dF2, psi_stvk_F, dpsi_stvk_dF, d2psi_stvk_dF2)
from . import meshes

__all__ = [n for n in dir() if not n.startswith("_")]
