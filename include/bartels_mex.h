/* bartels_mex.h - MATLAB-gateway facade of the GB300 library.
 *
 * The reference's MATLAB bindings are one mexFunction per routine
 * (matlab/<routine>.cpp, e.g. matlab/linear_tetmesh_neohookean_dq2.cpp:21-48):
 * each reads prhs[] with igl::matlab::parse_rhs_double / parse_rhs_index (the
 * latter subtracts 1, so E, q and fixed-vertex lists arrive 1-based), calls the
 * Eigen routine and returns the result with prepare_lhs_double (a dense result
 * as a column-major double matrix, a sparse one in MATLAB's compressed-column
 * arrays jc / ir / pr). bartels_mex_call does the same for every routine of the
 * tet and triangle families on the GPU behind one entry point, so that a single
 * gateway source, compiled once per routine name, replaces those files:
 *
 *   #include <mex.h>
 *   #include <bartels_mex.h>
 *   static int alloc(void *u, int64_t m, int64_t n, int64_t nnz, double **pr, uint64_t **ir, uint64_t **jc) {
 *     mxArray **out = (mxArray **)u;
 *     *out = nnz < 0 ? mxCreateDoubleMatrix(m, n, mxREAL) : mxCreateSparse(m, n, nnz > 0 ? nnz : 1, mxREAL);
 *     *pr = mxGetPr(*out);
 *     if (nnz >= 0) { *ir = (uint64_t *)mxGetIr(*out); *jc = (uint64_t *)mxGetJc(*out); }
 *     return 0;
 *   }
 *   void mexFunction(int nlhs, mxArray *plhs[], int nrhs, const mxArray *prhs[]) {
 *     bartels_mx in[16];
 *     for (int i = 0; i < nrhs && i < 16; ++i) in[i] = {(int64_t)mxGetM(prhs[i]), (int64_t)mxGetN(prhs[i]), mxGetPr(prhs[i])};
 *     if (bartels_mex_call(BARTELS_MEX_ROUTINE, nrhs, in, alloc, plhs)) mexErrMsgTxt(bartels_last_error());
 *   }
 *
 * built as `mex -DBARTELS_MEX_ROUTINE='"linear_tetmesh_neohookean_dq2"' gateway.cpp -lbartels_gpu`.
 *
 * Arguments, in the order of the reference's gateway for the routine:
 *   linear_tetmesh_dphi_dX(V, E)                          -> nT x 12
 *   linear_tetmesh_mass_matrix(V, E, densities, volumes)  -> sparse 3nV x 3nV
 *   fixed_point_constraint_matrix(V, fixed)               -> sparse d(nV - k) x d nV, d = size(V, 2)
 *   linear_tetmesh_<m>_q(V, E, q, dphidX, volumes, params)   -> 1 x 1,  m in neohookean, stvk, corotational, arap
 *   linear_tetmesh_<m>_dq(...)                               -> 3nV x 1
 *   linear_tetmesh_<m>_dq2(..., [psd])                       -> sparse; any 7th argument turns on
 *                                                              simple_psd_fix with tolerance 1e-3
 *   linear_tetmesh_linear_elasticity_dq2(V, E, q, dphidX, volumes, params)  (params = Young's modulus, Poisson ratio)
 *   linear_tri2dmesh_dphi_dX(V, E)                        -> nT x 6     (V nV x 2)
 *   linear_tri2dmesh_mass_matrix(V, E, densities, areas)  -> sparse 2nV x 2nV
 *   linear_tri2dmesh_<m>_{q,dq,dq2}(V, E, q, dphidX, areas, params[, psd]), linear_tri2dmesh_linear_elasticity_dq2
 *   linear_tri3dmesh_dphi_dX(V, E)                        -> nT x 9
 *   linear_tri3dmesh_stvk_dq2(V, E, q, dphidX, N, n, dndq, areas, params[, psd])  -> sparse 3nV x 3nV
 *   dpsi_neohookean_dF(E, F, params)                      -> 9nT x 1 (F nT x 9, row t = flatten of F_t)
 *   d2psi_neohookean_dF2(E, F, params), d2psi_stvk_dF2    -> sparse 9nT x 9nT, block diagonal
 *
 * E and fixed are 1-based doubles as MATLAB passes them; they must be integral
 * and in range (the reference's gateways do not check). q is used as given: the
 * gateways' parse_rhs_index also subtracts 1 from every coordinate of q, a rigid
 * translation that none of these energies, gradients or Hessians depends on
 * (the shape-function gradients of an element sum to zero), so the results
 * agree up to rounding; leaving q alone keeps the FP32 displacement path of the
 * tet Hessian at full precision. Sparse results keep the assembled pattern,
 * the structural zeros included, column by column with ascending rows
 * (setFromTriplets' pattern), each value H(ir[k], column) exactly as assembled.
 * Precision is that of the C ABI entry point behind each routine (tet Hessian
 * and mass values: FP32 element math; everything else FP64).
 *
 * The facade keeps one context on device 0 and caches mesh plans by content
 * (V and E for tets, E for triangles; the four most recently used), so repeated
 * calls on one mesh skip pattern construction. Calls are serialised by a
 * mutex. Returns a BARTELS_* status; bartels_last_error() has the message. */
#ifndef BARTELS_MEX_H
#define BARTELS_MEX_H

#include <stdint.h>

#include "bartels_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* A real double matrix as mexFunction receives it: m x n, column-major. */
typedef struct {
  int64_t m, n;
  const double *pr;
} bartels_mx;

/* Output allocation. nnz < 0: create a dense m x n double matrix and set *pr.
 * nnz >= 0: create an m x n sparse matrix with room for nnz entries and set
 * *pr (nnz values), *ir (nnz row indices) and *jc (n + 1 column starts), the
 * indices being 64-bit (mwIndex). Return 0 on success. */
typedef int (*bartels_mx_alloc)(void *user, int64_t m, int64_t n, int64_t nnz, double **pr, uint64_t **ir,
                                uint64_t **jc);

int bartels_mex_call(const char *routine, int nrhs, const bartels_mx *prhs, bartels_mx_alloc alloc, void *user);
/* The routines bartels_mex_call accepts. */
int bartels_mex_routine_count(void);
const char *bartels_mex_routine_name(int i);
/* Release the facade's cached plans and context (for mexAtExit). */
void bartels_mex_release(void);

#ifdef __cplusplus
}
#endif
#endif /* BARTELS_MEX_H */
