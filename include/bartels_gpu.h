/* bartels_gpu.h -- C ABI of the GB300 (sm_103a) implementation of the
 * tet-mesh hyperelastic path of dilevin/Bartels.
 *
 * Plain C: pointers and sizes only, no C++ or torch types. Every function
 * returns an int status (BARTELS_OK = 0). Nothing calls exit(); a failed call
 * leaves its outputs unspecified and bartels_last_error() describes it.
 *
 * Conventions (the reference's, see the Bartels sources cited per function):
 *   V       nV x 3 double, column-major (all x, then y, then z)
 *   E       nT x 4 int, column-major, 0-based
 *   q, g    3 nV double, interleaved [x0 y0 z0 x1 ...]
 *   dphidX  nT x 12 double, column-major; row t = column-major flatten of the
 *           4x3 matrix of shape-function gradients of tet t
 *   volume  nT double
 *   params  nT x 2 double, column-major; Neo-Hookean (C, D) = (mu/2, lambda/2),
 *           StVK and corotational (lambda, mu)
 *   sparse  CSR of the symmetric 3nV x 3nV matrix. Its pattern is the full 3x3
 *           block pattern of the mesh graph (every vertex pair sharing a tet, the
 *           vertex itself included), which is exactly the pattern that the
 *           reference's sim::assemble produces (explicit zeros kept). Because the
 *           pattern is symmetric the CSR arrays are also the reference's CSC.
 *
 * Host-pointer entry points copy inputs to the GPU, compute on the context's
 * stream and copy results back before returning. The *_d variants take device
 * pointers and only enqueue work on the context's stream.
 */
#ifndef BARTELS_GPU_H
#define BARTELS_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status --- */
enum {
  BARTELS_OK = 0,
  BARTELS_E_INVALID_ARG = 1,
  BARTELS_E_NONFINITE = 2,     /* an element produced NaN/Inf (e.g. J <= 0 for Neo-Hookean) */
  BARTELS_E_NOT_CONVERGED = 3, /* PCG or Newton hit its iteration cap */
  BARTELS_E_DEVICE = 4,        /* CUDA error */
  BARTELS_E_TIMEOUT = 5,
  BARTELS_E_UNSUPPORTED = 6,   /* mesh outside the kernels' limits (e.g. > 255 neighbours) */
  BARTELS_E_NO_DEVICE = 7
};

/* Exit status of line search / Newton, include/BartelsTypes.h:6-9. */
enum { BARTELS_CONVERGED = 0, BARTELS_MAX_ITERATIONS_REACHED = 1 };

/* Material laws. NEOHOOKEAN is src/psi_neohookean_F.cpp:31 (C (I1-3-2 ln J) +
 * D (J-1)^2). NEOHOOKEAN_ISOCHORIC is the reference's earlier law kept as
 * commented-out code in src/psi_neohookean_F.cpp:8-14 (C (J^-2/3 I1 - 3) +
 * D (J-1)^2); data/matrices/H_neohookean_coarser_bunny.txt was made with it.
 * ARAP is src/psi_arap_S.cpp:8-11 (k sum (s_i - 1)^2 over the singular values,
 * params column 0 = k; Hessian in the reference's stretch layout, as the
 * corotational model). LINEAR_ELASTICITY is src/linear_tet_linear_elasticity_dq2.cpp
 * (B^T C B vol, Voigt engineering strains of e = sym(F) of q as given, so q is
 * a displacement; params = Young's modulus, Poisson ratio at the host entry
 * points; a plan's stored params for this model, as the device entry points
 * read them, are the Lame pair (lambda, mu)). Its energy, mu e:e +
 * lambda/2 tr(e)^2, has no reference counterpart; its gradient B^T C e vol
 * follows src/linear_tet_linear_elasticity_dq.cpp, which would not compile if
 * instantiated (a 6x12 product stored in a 9x12 matrix). */
enum {
  BARTELS_NEOHOOKEAN = 0,
  BARTELS_STVK = 1,
  BARTELS_COROTATIONAL = 2,
  BARTELS_NEOHOOKEAN_ISOCHORIC = 3,
  BARTELS_ARAP = 4,
  BARTELS_LINEAR_ELASTICITY = 5
};

/* Element-matrix callback replacement (src/linear_tetmesh_neohookean_dq2.cpp:22):
 * a host functor cannot run on the GPU, so the one callback the reference uses,
 * simple_psd_fix (src/simple_psd_fix.cpp:5-21), is selected by flag. */
enum { BARTELS_PSD_NONE = 0, BARTELS_PSD_SIMPLE_FIX = 1 };

/* Flags for the dq2 entry points. */
enum {
  /* corotational only: use the exact Hessian instead of the reference's layout.
   * The reference (src/d2psi_stretch_dF2.cpp:37-45) fills d2psi/dF2 in row-major
   * F order while B is column-major, so its matrix is the Hessian at F^T; that
   * is the default here, for drop-in parity. */
  BARTELS_DQ2_COROT_EXACT = 1
};

typedef struct bartels_ctx_s *bartels_ctx;
typedef struct bartels_mesh_plan_s *bartels_mesh_plan;

const char *bartels_status_string(int status);
/* Text of the last error raised on the calling thread ("" if none). */
const char *bartels_last_error(void);

/* ---------------------------------------------------------------- context -- */
/* One context per host thread: a device, a stream, workspace and a pinned
 * staging area. All work is ordered on the context's stream. No counterpart
 * in the reference (single-threaded host code, include/EigenTypes.h:133-135
 * holds its only globals). */
int bartels_ctx_create(int device, bartels_ctx *out);
/* Destroy every plan created on ctx before destroying ctx. */
int bartels_ctx_destroy(bartels_ctx ctx);
int bartels_ctx_synchronize(bartels_ctx ctx);
/* The context's cudaStream_t, as void*. */
void *bartels_ctx_stream(bartels_ctx ctx);
/* Number of kernels this library enqueued on ctx since creation. */
int64_t bartels_ctx_kernel_launches(bartels_ctx ctx);

/* ------------------------------------------------------------- kinematics -- */
/* linear_tetmesh_dphi_dX, src/linear_tetmesh_dphi_dX.cpp:5-18 (per tet:
 * src/linear_tet_dphi_dX.cpp:10-16). dphidX: nT x 12 column-major. */
int bartels_tetmesh_dphi_dX(bartels_ctx ctx, int nV, const double *V, int nT, const int *E, double *dphidX);
/* Signed tet volumes det[X1-X0, X2-X0, X3-X0]/6 (the reference's callers use
 * igl::volume, tests/test_constitutive_model.cpp:28). */
int bartels_tetmesh_volume(bartels_ctx ctx, int nV, const double *V, int nT, const int *E, double *vol);

/* ------------------------------------------------------------------ plan --- */
/* A mesh plan is built once from (V, E): rest data, per-tet records, the
 * vertex->tet incidence lists in tet order, the block CSR pattern and the
 * element->CSR scatter positions. The reference has no counterpart: it
 * rebuilds its triplets and pattern in every assemble call
 * (src/assemble.cpp:57-94); the plan keeps that pattern, bit-exact. Plans are immutable after creation apart from
 * the element data set with bartels_plan_set_element_data. */
int bartels_plan_create(bartels_ctx ctx, int nV, const double *V, int nT, const int *E, bartels_mesh_plan *out);
int bartels_plan_destroy(bartels_mesh_plan plan);
/* Upload per-tet element data (host pointers; any may be NULL to keep the
 * plan's current values). Defaults after plan creation: dphidX and volume
 * computed from V, params = 0, density = 0. */
int bartels_plan_set_element_data(bartels_mesh_plan plan, const double *dphidX, const double *vol,
                                  const double *params, const double *density);
/* Scalar CSR size of the 3nV x 3nV pattern. */
int bartels_plan_csr_size(bartels_mesh_plan plan, int *n, int64_t *nnz);
/* Host copy of the CSR pattern: row_ptr (n+1), col_idx (nnz). */
int bartels_plan_csr_pattern(bartels_mesh_plan plan, int *row_ptr, int *col_idx);

/* ------------------------------------------------------ energy / gradient -- */
/* linear_tetmesh_{neohookean,stvk,corotational}_q, e.g.
 * src/linear_tetmesh_neohookean_q.cpp:10-24: sum over tets of psi(F) vol.
 * dphidX/vol/params may be NULL to use the plan's element data; otherwise they
 * are uploaded first (as bartels_plan_set_element_data). FP64 element math,
 * deterministic FP64 reduction. */
int bartels_tetmesh_q(bartels_ctx ctx, bartels_mesh_plan plan, int model, const double *q, const double *dphidX,
                      const double *vol, const double *params, double *energy);
/* linear_tetmesh_{model}_dq, e.g. src/linear_tetmesh_neohookean_dq.cpp:5-22:
 * assembled gradient g (3 nV). FP64 element math, per-vertex sums in tet order. */
int bartels_tetmesh_dq(bartels_ctx ctx, bartels_mesh_plan plan, int model, const double *q, const double *dphidX,
                       const double *vol, const double *params, double *g);
/* linear_tetmesh_{model}_dq2, e.g. src/linear_tetmesh_neohookean_dq2.cpp:8-28:
 * assembled Hessian values in the plan's CSR order (nnz doubles). FP32 element
 * math; each entry summed over its tets in tet order (the order in which the
 * reference's setFromTriplets sums duplicates). psd_mode/psd_tol replace the
 * element callback; flags: BARTELS_DQ2_*. */
int bartels_tetmesh_dq2(bartels_ctx ctx, bartels_mesh_plan plan, int model, const double *q, const double *dphidX,
                        const double *vol, const double *params, int psd_mode, double psd_tol, int flags,
                        double *csr_values);

/* Named drop-ins, the reference's linear_tetmesh_<model>_{q,dq,dq2}
 * (include/linear_tetmesh_neohookean_q.h:13-18, _dq.h:13-17, _dq2.h:14-21 and the
 * StVK, corotational, ARAP and linear-elasticity siblings): the generic calls
 * with the model fixed. */
int bartels_tetmesh_neohookean_q(bartels_ctx, bartels_mesh_plan, const double *q, const double *dphidX,
                                 const double *vol, const double *params, double *energy);
int bartels_tetmesh_neohookean_dq(bartels_ctx, bartels_mesh_plan, const double *q, const double *dphidX,
                                  const double *vol, const double *params, double *g);
int bartels_tetmesh_neohookean_dq2(bartels_ctx, bartels_mesh_plan, const double *q, const double *dphidX,
                                   const double *vol, const double *params, int psd_mode, double psd_tol,
                                   double *csr_values);
int bartels_tetmesh_stvk_q(bartels_ctx, bartels_mesh_plan, const double *q, const double *dphidX,
                           const double *vol, const double *params, double *energy);
int bartels_tetmesh_stvk_dq(bartels_ctx, bartels_mesh_plan, const double *q, const double *dphidX,
                            const double *vol, const double *params, double *g);
int bartels_tetmesh_stvk_dq2(bartels_ctx, bartels_mesh_plan, const double *q, const double *dphidX,
                             const double *vol, const double *params, int psd_mode, double psd_tol,
                             double *csr_values);
int bartels_tetmesh_corotational_q(bartels_ctx, bartels_mesh_plan, const double *q, const double *dphidX,
                                   const double *vol, const double *params, double *energy);
int bartels_tetmesh_corotational_dq(bartels_ctx, bartels_mesh_plan, const double *q, const double *dphidX,
                                    const double *vol, const double *params, double *g);
int bartels_tetmesh_corotational_dq2(bartels_ctx, bartels_mesh_plan, const double *q, const double *dphidX,
                                     const double *vol, const double *params, int psd_mode, double psd_tol,
                                     double *csr_values);
/* linear_tetmesh_arap_{q,dq,dq2}, src/linear_tetmesh_arap_q.cpp, _dq.cpp, _dq2.cpp */
int bartels_tetmesh_arap_q(bartels_ctx, bartels_mesh_plan, const double *q, const double *dphidX,
                           const double *vol, const double *params, double *energy);
int bartels_tetmesh_arap_dq(bartels_ctx, bartels_mesh_plan, const double *q, const double *dphidX,
                            const double *vol, const double *params, double *g);
int bartels_tetmesh_arap_dq2(bartels_ctx, bartels_mesh_plan, const double *q, const double *dphidX,
                             const double *vol, const double *params, int psd_mode, double psd_tol,
                             double *csr_values);
/* linear_tetmesh_linear_elasticity_{dq,dq2}, src/linear_tetmesh_linear_elasticity_dq.cpp,
 * _dq2.cpp (the energy entry point has no reference counterpart) */
int bartels_tetmesh_linear_elasticity_q(bartels_ctx, bartels_mesh_plan, const double *q, const double *dphidX,
                                        const double *vol, const double *params, double *energy);
int bartels_tetmesh_linear_elasticity_dq(bartels_ctx, bartels_mesh_plan, const double *q, const double *dphidX,
                                         const double *vol, const double *params, double *g);
int bartels_tetmesh_linear_elasticity_dq2(bartels_ctx, bartels_mesh_plan, const double *q, const double *dphidX,
                                          const double *vol, const double *params, int psd_mode, double psd_tol,
                                          double *csr_values);

/* --------------------------------------------------------- pointwise laws -- */
/* The laws themselves over n deformation gradients: psi_<law>_F,
 * dpsi_<law>_dF and d2psi_<law>_dF2 of the reference (src/psi_neohookean_F.cpp:31,
 * src/dpsi_neohookean_dF.cpp:58-66, src/d2psi_neohookean_dF2.cpp:185-283,
 * src/psi_stvk_F.cpp, src/dpsi_stvk_dF.cpp, src/d2psi_stvk_dF2.cpp; the
 * corotational and ARAP laws through src/psi_stretch_F.cpp, src/dpsi_stretch_dF.cpp
 * and src/d2psi_stretch_dF2.cpp, in the reference's layout). F: n x 9
 * column-major, row t the column-major flatten [F11 F21 F31 F12 ...] of F_t;
 * params n x 2 column-major (the mesh entry points' per-tet rows, volume 1).
 * Outputs (any may be NULL): psi n; dpsi n x 9 column-major, row t = dpsi/dF in
 * the same flatten; d2psi n blocks of 81, block t the column-major 9 x 9 with
 * entry (r, c) = d2psi / dvec(F)_r dvec(F)_c. FP64 on the device. */
int bartels_pointwise_laws(bartels_ctx ctx, int model, int n, const double *F, const double *params, double *psi,
                           double *dpsi, double *d2psi);

/* --------------------------------------------------- mass, loads, bounds --- */
/* linear_tetmesh_mass_matrix, src/linear_tetmesh_mass_matrix.cpp:7-24 (per tet
 * src/linear_tet_mass_matrix.cpp:12-42): values in the plan's CSR order. */
int bartels_tetmesh_mass_matrix(bartels_ctx ctx, bartels_mesh_plan plan, const double *density, const double *vol,
                                double *csr_values);
/* assemble (src/assemble.cpp:36-97), the reference's generic assembler, for
 * element quantities the caller computed (its element functor cannot run on
 * the device): Ke holds nT blocks of 144 doubles, block t the column-major
 * 12 x 12 with row / column 3a + k for local vertex a and coordinate k; the
 * values are summed per CSR entry in tet order, the order in which
 * setFromTriplets sums the reference's duplicate triplets, so the FP64 result
 * is the reference's bit for bit. Output in the plan's CSR order. */
int bartels_plan_assemble_matrix(bartels_ctx ctx, bartels_mesh_plan plan, const double *Ke, double *csr_values);
/* Vector form (src/assemble.cpp:100-132): ge nT x 12 element-major (entry
 * 12 t + 3a + k), summed per vertex in tet order into g (3nV). */
int bartels_plan_assemble_vector(bartels_ctx ctx, bartels_mesh_plan plan, const double *ge, double *g);
/* linear_tetmesh_const_ext_force, src/linear_tetmesh_const_ext_force.cpp:5-18:
 * f_v = sum over tets of v of vol/4 * traction. */
int bartels_tetmesh_const_ext_force(bartels_ctx ctx, bartels_mesh_plan plan, const double *vol,
                                    const double traction[3], double *f);
/* fixed_point_constraint_matrix, src/fixed_point_constraint_matrix.cpp:7-38.
 * fixed (sorted ascending, as the reference requires). Rows = dim*(nV-nfix),
 * cols = dim*nV, one 1 per row: row_ptr (rows+1), col_idx (rows), values all 1.
 * Host-side (integer bookkeeping only). Pass row_ptr = NULL to query rows. */
int bartels_fixed_point_constraint_matrix(int nV, int dim, const int *fixed, int nfix, int *rows, int *row_ptr,
                                          int *col_idx, double *values);
/* find_min_vertices, src/find_min_vertices.cpp:5-21: indices of vertices whose
 * coordinate dim is within tol of the minimum. Returns count in *count. */
int bartels_find_min_vertices(int nV, const double *V, int dim, double tol, int *indices, int *count);

/* ------------------------------------------------------------ linear solve -- */
typedef struct {
  double rel_tol;       /* relative residual target ||b - A x|| / ||b|| (default 1e-8) */
  int max_iters;        /* total PCG iterations cap (default 20000) */
  double inner_rel_tol; /* FP32 inner PCG: reduction of the residual per refinement pass (default 0.1) */
  int max_refinements;  /* residual refinement passes (default 40); the refinement residual is
                           float-float (~2^-48 relative) on the block layout, FP64 on a CSR */
  int restart;          /* 0 (default): each refinement pass replaces the FP32 residual by the FP64 one
                           b - A x and continues the previous pass's search direction (reliable update,
                           one replacement per 10x reduction by default); 1: each pass restarts the inner
                           PCG from p = 0 (pair with inner_rel_tol about 1e-4) */
} bartels_pcg_params;

typedef struct {
  int iterations;      /* total PCG iterations */
  int refinements;     /* FP64 refinement passes used */
  double rel_residual; /* final ||b - A x|| / ||b|| in FP64 */
  int converged;
} bartels_pcg_report;

void bartels_pcg_default_params(bartels_pcg_params *p);

/* search_direction_newton_sparse, src/search_direction_newton_sparse.cpp:5-26:
 * d = -H^{-1} g for an SPD H given as CSR (host arrays, nnz values double).
 * Replaces the reference's Eigen::SparseLU with block-Jacobi PCG (FP32 with
 * float-float residual refinement). n must be a multiple of 3 for the 3x3 block
 * preconditioner (falls back to scalar Jacobi otherwise). Returns
 * BARTELS_E_NOT_CONVERGED where the reference's solver.info() != Success. */
int bartels_search_direction_newton_sparse(bartels_ctx ctx, int n, const int *row_ptr, const int *col_idx,
                                           const double *values, const double *g, double *d,
                                           const bartels_pcg_params *params, bartels_pcg_report *report);

/* ------------------------------------------------------------- line search -- */
/* linesearch_backtracking_bisection, src/linesearch_backtracking_bisection.cpp:5-31,
 * for a host objective: while f(x + alpha d) > f(x) + c g.d and it < max_it:
 * alpha *= p. Then x += alpha d. *status = BARTELS_CONVERGED or
 * BARTELS_MAX_ITERATIONS_REACHED, exactly as the reference. The vector update
 * and dot product run on the host arrays given (this entry point exists for
 * callers with their own host objective; the GPU Newton solver below runs its
 * line search on the device). */
typedef double (*bartels_objective_fn)(const double *x, int n, void *user);
int bartels_linesearch_backtracking_bisection(int n, double *x, const double *d, bartels_objective_fn f,
                                              void *user, const double *g, int max_iterations, double alpha,
                                              double c, double p, int *status, double *alpha_out);

/* ------------------------------------------------------------------ Newton -- */
/* Objective minimised by bartels_newton_solve over the unknown x (3 nV):
 *   q(x)  = q_base + scale * x
 *   f(x)  = mass_coeff * (1/2 x^T M x - x^T M x_hat) + Psi(q(x)) - force_scale * x^T f_ext
 * restricted to the free vertices (pinned vertices keep x = 0).
 * Quasi-static (Newton under gravity): mass_coeff 0, scale 1, q_base 0.
 * Implicit Euler in velocity form (matlab/examples/implicit_integration.m:69-83):
 *   x = v, q_base = q_t, scale = dt, x_hat = v_t, force_scale = dt, mass_coeff 1.
 * M is the consistent mass matrix of the plan's density. */
typedef struct {
  int model;
  int psd_mode;          /* BARTELS_PSD_* for the Hessian */
  double psd_tol;
  int dq2_flags;
  double mass_coeff;
  double scale;
  double force_scale;
  /* Newton (include/optimization_gradient_based.h:51-56 defaults) */
  double gradient_tol;   /* absolute tol (reference) when relative == 0, else relative */
  int relative;          /* 1: stop when ||g|| <= gradient_tol * ||g_0|| */
  int max_iterations;    /* reference: loop runs while iteration_count <= max_iterations */
  int max_iterations_ls;
  double ls_alpha, ls_c, ls_p;
  bartels_pcg_params pcg;
} bartels_newton_params;

typedef struct {
  int status;            /* BARTELS_CONVERGED / BARTELS_MAX_ITERATIONS_REACHED */
  int iterations;        /* Newton iterations taken */
  int pcg_iterations;    /* total PCG iterations */
  int ls_iterations;     /* total line-search backtracks */
  int ls_failures;       /* line searches that hit max_iterations_ls */
  double grad_norm0, grad_norm;
  double energy;
  double seconds;        /* wall time of the solve (device-synchronised) */
  double t_gradient, t_hessian, t_pcg, t_linesearch; /* seconds per stage, summed */
  /* last Newton iteration */
  double last_alpha;             /* accepted line-search step */
  double last_pcg_rel_residual;  /* FP64 ||b - A d|| / ||b|| of the search direction */
  int last_pcg_iterations;
  int last_pcg_refinements;
  int pcg_failures;              /* searches whose PCG did not reach rel_tol */
  double energy_change;          /* f(x_new) - f(x_old) of the last step */
  int precond_fallbacks;         /* learned-preconditioner solves redone with block-Jacobi */
  double t_precond;              /* seconds spent building the learned factor */
} bartels_newton_report;

void bartels_newton_default_params(bartels_newton_params *p);

/* Problem data for a Newton solve on a plan (host pointers; may be NULL):
 * q_base (3nV), x_hat (3nV), f_ext (3nV), pinned (nV bytes, 1 = vertex fixed). */
int bartels_newton_set_problem(bartels_mesh_plan plan, const double *q_base, const double *x_hat,
                               const double *f_ext, const unsigned char *pinned);
/* newtons_method_bisection (include/optimization_gradient_based.h:43-110) on the
 * objective above: gradient test (relative, or the reference's absolute one),
 * Hessian, search direction, line search, until converged or max_iterations.
 * Solve from x (host, 3nV, in/out). Host buffers, copies counted in the time. */
int bartels_newton_solve(bartels_ctx ctx, bartels_mesh_plan plan, const bartels_newton_params *params,
                         double *x, bartels_newton_report *report);
/* Device-resident variant: x_d is a device pointer (3nV doubles). */
int bartels_newton_solve_d(bartels_ctx ctx, bartels_mesh_plan plan, const bartels_newton_params *params,
                           double *x_d, bartels_newton_report *report);
/* One Newton iteration (gradient, Hessian, PCG, line search) on device x_d;
 * *done = 1 when the gradient test passed before the step. Used by benchmarks
 * that time individual iterations. g0_norm: reference gradient norm for the
 * relative test (<= 0 to compute it now). */
int bartels_newton_iterate_d(bartels_ctx ctx, bartels_mesh_plan plan, const bartels_newton_params *params,
                             double *x_d, double g0_norm, int *done, bartels_newton_report *report);

/* Gradient of the Newton objective at device x_d into g_d (3nV, rows of pinned
 * vertices 0): the residual the Newton step solves against. */
int bartels_newton_gradient_d(bartels_ctx ctx, bartels_mesh_plan plan, const bartels_newton_params *params,
                              const double *x_d, double *g_d);

/* Copy the plan's current q_base and x_hat (host, 3nV doubles each; either may
 * be NULL) back, e.g. after bartels_newton_advance_implicit_euler_d moved them
 * on the device. A state accessor with no counterpart in the reference. */
int bartels_newton_get_problem(bartels_mesh_plan plan, double *q_base, double *x_hat);

/* Value of the Newton objective at device x_d (FP64, host *energy): the
 * function f that newtons_method_bisection minimises and its line search
 * evaluates (include/optimization_gradient_based.h:77-106; here the
 * implicit-Euler objective of matlab/examples/implicit_integration.m:69-83,
 * f = mass_coeff (x^T M x / 2 - x^T M x_hat) + Psi(q_base + scale x)
 * - force_scale x^T f_ext over the free vertices). */
int bartels_newton_energy_d(bartels_ctx ctx, bartels_mesh_plan plan, const bartels_newton_params *params,
                            const double *x_d, double *energy);

/* --------------------------------------------------- learned preconditioner -- */
/* No counterpart in the reference, whose linear solver is Eigen::SparseLU
 * (include/search_direction_newton_sparse.h:8). A message-passing network over
 * the mesh vertex graph outputs a block-lower-triangular factor G on the
 * Hessian's pattern; PCG uses M^-1 = G^T G (two triangular gathers, no
 * triangular solves). With its output layers at zero the factor is the 3x3
 * block-Jacobi one. It is trained on the GPU (forward, backward and Adam in
 * this library) to minimise log of Kaporin's condition number of G H G^T,
 * estimated with probe vectors, on Hessians the Newton solver produces. */
typedef struct bartels_lpcg_s *bartels_lpcg;
enum {
  BARTELS_PRECOND_BLOCK_JACOBI = 0,
  BARTELS_PRECOND_LEARNED = 1,            /* M^-1 = G^T G, the network's factor */
  BARTELS_PRECOND_MULTIGRID = 2,          /* aggregation multigrid V-cycle, block-Jacobi smoothing */
  BARTELS_PRECOND_LEARNED_MULTIGRID = 3   /* the same V-cycle with the network's G^T G as fine smoother */
};

int bartels_lpcg_create(bartels_ctx ctx, bartels_lpcg *out);
int bartels_lpcg_destroy(bartels_lpcg net);
/* number of FP32 parameters (flat vector; layout in bartels_gb300/lpcg.py) */
int bartels_lpcg_num_params(void);
int bartels_lpcg_set_params(bartels_lpcg net, const float *params);
/* params and/or grad (host, num_params floats each; either may be NULL) */
int bartels_lpcg_get_params(bartels_lpcg net, float *params, float *grad);
/* One training step on a plan's Hessian (values_d: FP32, the plan's CSR order,
 * device; pinned vertices from bartels_newton_set_problem). Probes: nprobes
 * Rademacher vectors from seed, plus residual_d (device, 3nV FP64) when not
 * NULL. Computes the loss and the parameter gradient; lr > 0 also applies
 * one Adam step (gradient clipped to norm clip when clip > 0). */
int bartels_lpcg_train_step(bartels_lpcg net, bartels_mesh_plan plan, const float *values_d,
                            const double *residual_d, int nprobes, unsigned seed, float lr, float clip,
                            double *loss);
/* Network outputs for the plan's Hessian values_d: raw (host, 9 per lower block:
 * the 3x3 Ghat block, or d0..d5 at the diagonal) and G in lower storage (host,
 * 9 per lower block, three scalar rows per vertex). Either may be NULL. */
int bartels_lpcg_outputs(bartels_lpcg net, bartels_mesh_plan plan, const float *values_d, float *raw,
                         float *g_lower);
/* Number of lower (j <= v) and upper (j >= v) blocks of the plan's pattern. */
int bartels_plan_factor_size(bartels_mesh_plan plan, int64_t *nnzl_blocks, int64_t *nnzu_blocks);
/* Preconditioner of the plan's PCG solves (Newton and bartels_plan_pcg_d):
 * BARTELS_PRECOND_BLOCK_JACOBI; BARTELS_PRECOND_LEARNED with net;
 * BARTELS_PRECOND_MULTIGRID (net ignored): one V-cycle of aggregation
 * multigrid per PCG iteration (greedy aggregates of the free vertices, the
 * six rigid-body modes per aggregate as the tentative prolongator, Galerkin
 * coarse levels, Chebyshev smoothing, a dense coarsest solve; the hierarchy
 * is built on the first solve and again whenever the pinned set changes);
 * BARTELS_PRECOND_LEARNED_MULTIGRID with net: the same V-cycle with the
 * network's M = G^T G as the smoother of the finest level. Block-Jacobi is
 * the fallback when a learned or multigrid solve does not converge, and the
 * preconditioner of systems too small for a coarse level. No counterpart in
 * the reference (its solver is Eigen::SparseLU). */
int bartels_plan_set_preconditioner(bartels_mesh_plan plan, int kind, bartels_lpcg net);
/* Shape of the plan's multigrid hierarchy (built by the last multigrid solve
 * or bartels_plan_precond_apply_d): *levels, and for each of the first
 * max_levels levels its nodes (vertices on level 0, aggregates below) and
 * stored blocks (3x3 on level 0, 6x6 below); *coarsest is 0 for a dense
 * coarsest solve, 1 for an exact block-diagonal one, 2 for Chebyshev
 * smoothing. Arrays may be NULL. BARTELS_E_INVALID_ARG without a hierarchy.
 * No counterpart in the reference. */
int bartels_plan_mg_info(bartels_mesh_plan plan, int max_levels, int *levels, int *nodes, int64_t *blocks,
                         int *coarsest);
/* z_d = B r_d: one application of the plan's multigrid preconditioner
 * (BARTELS_PRECOND_MULTIGRID or _LEARNED_MULTIGRID) built for the Hessian
 * values_d (FP32, the plan's CSR order, device); FP32 device vectors of 3nV,
 * rows of pinned vertices zero. For tests of the preconditioner itself
 * (symmetry, positivity). levels (host, may be NULL) receives the number of
 * levels. No counterpart in the reference. */
int bartels_plan_precond_apply_d(bartels_ctx ctx, bartels_mesh_plan plan, const float *values_d, const float *r_d,
                                 float *z_d, int *levels);
/* x_d = H^-1 b_d by PCG on the plan's Hessian (values_d, or NULL for the plan's
 * internal Hessian buffer) with the plan's preconditioner; device FP64 vectors,
 * rows of pinned vertices excluded. */
int bartels_plan_pcg_d(bartels_ctx ctx, bartels_mesh_plan plan, const float *values_d, const double *b_d,
                       double *x_d, const bartels_pcg_params *params, bartels_pcg_report *report);
/* ---------------------------------------------------------------- batching -- */
/* Autotuner: times the PCG loop's block-row SpMV (4, 8, 16 lanes per vertex row) and the
 * factor passes (4, 8 lanes) on this plan's Hessian (values_d, or NULL for the
 * plan's internal buffer) and keeps the fastest for the plan's PCG solves. The
 * choice is cached in the context per size bucket floor(log2 nV) and reused by
 * later plans of that bucket unless force != 0. No counterpart in the reference. */
int bartels_plan_autotune(bartels_ctx ctx, bartels_mesh_plan plan, const float *values_d, int force,
                          int *spmv_lanes, int *factor_lanes);
/* The PCG loop's SpMV kernel, y_d = A x_d with A the FP32 values_d (NULL:
 * the plan's last assembled Hessian), timed: 3 warm-up launches, then reps
 * launches between CUDA events on the context's stream; *us_per_launch gets
 * the mean. The loop reads a copy of the values whose scalar rows are padded
 * to multiples of 4 entries (4 values per 16-byte load); the copy is made
 * here once, as the solver makes it once per linear solve (environment
 * BARTELS_PCG_PADDED=0 keeps the values' own layout). For measurement; no
 * counterpart in the reference. */
int bartels_plan_pcg_spmv_time_d(bartels_ctx ctx, bartels_mesh_plan plan, const float *values_d, const float *x_d,
                                 float *y_d, int reps, double *us_per_launch);

/* Hessian autotuner: times the fused simple_psd_fix-projected assembly of the
 * plan at device positions q_d for the assembly's CTA shapes (128 vertices
 * per CTA with 64 KB of shared memory, or 64 vertices with 32 KB) and the PSD
 * pre-pass block sizes (64, 128, 256 threads), keeps the fastest pair for the
 * plan's Hessians and caches it in the context per size bucket floor(log2 nV)
 * (reused by later plans of that bucket unless force != 0). The assembled
 * values do not depend on the choice. No counterpart in the reference. */
int bartels_plan_autotune_hessian(bartels_ctx ctx, bartels_mesh_plan plan, int model, const double *q_d, int force,
                                  int *chunk_vertices, int *psd_block);
/* Set the same choice by hand (chunk_vertices 64 or 128, psd_block 64, 128
 * or 256). */
int bartels_plan_set_hessian_tuning(bartels_mesh_plan plan, int chunk_vertices, int psd_block);
/* Batched solves pack many meshes into one plan (a block-diagonal system, one
 * launch per Newton stage for all of them); per-mesh convergence uses
 * out_d[s] = sum of v_d^2 over the DOFs of vertices vertex_offsets_d[s] ..
 * vertex_offsets_d[s+1]-1 (device arrays, nseg + 1 offsets). */
int bartels_segment_sumsq_d(bartels_ctx ctx, int nseg, const int *vertex_offsets_d, const double *v_d,
                            double *out_d);
/* Declare the plan's mesh as nseg independent packed meshes (segments):
 * vertex_offsets (nseg + 1) and tet_offsets (nseg + 1), host arrays, every
 * tet's vertices inside its own segment's range. The plan's PCG solves then
 * keep separate scalars per segment (alpha, beta, r.z, convergence against
 * the segment's own residual target), and the Newton line search backtracks
 * each segment on its own energy difference with its own step, so that each
 * packed mesh follows the iterates it would follow alone (the reference runs
 * one newtons_method_bisection per problem,
 * include/optimization_gradient_based.h:77-106, each with its own
 * linesearch_backtracking_bisection, src/linesearch_backtracking_bisection.cpp:17-30).
 * The preconditioners (block-Jacobi, multigrid) are block diagonal over the
 * segments already. nseg = 0 returns to one system. Every segment starts
 * active. */
int bartels_plan_set_segments(bartels_mesh_plan plan, int nseg, const int *vertex_offsets,
                              const int64_t *tet_offsets);
/* Segments with active[s] = 0 (host, nseg bytes) take no Newton step and no
 * PCG iteration (their search direction is 0), e.g. instances that have met
 * their convergence test. */
int bartels_plan_set_segment_active(bartels_mesh_plan plan, const unsigned char *active);
/* PCG iterations each segment took in the plan's last solve (host, nseg). */
int bartels_plan_segment_pcg_iterations(bartels_mesh_plan plan, int *iterations);
/* Building block: Y = act(X W^T + bias) on the tensor cores (tcgen05, TMA);
 * X: M x K BF16 (row stride ldx elements), W: N x K BF16, bias: N FP32 or NULL,
 * Y: M x N FP32 (row stride ldy); N, K in {64, 128}; device pointers. */
int bartels_gemm_bf16_d(bartels_ctx ctx, int M, int N, int K, const void *x_d, int ldx, const void *w_d,
                        const float *bias_d, int relu, float *y_d, int ldy);
/* Failure-path probe of the same tensor-core GEMM (for tests): every CTA
 * issues no copy and no MMA and polls its first mbarrier, which nothing
 * arrives on, `polls` times; the bounded wait runs out and the kernel takes
 * its time-out path (error flag set, no output written, tensor memory freed),
 * which this call reports as BARTELS_E_TIMEOUT like a real time-out. Nothing
 * is in flight when the wait gives up. No counterpart in the reference. */
int bartels_gemm_bf16_wait_probe_d(bartels_ctx ctx, int M, int N, int K, const void *x_d, int ldx,
                                   const void *w_d, float *y_d, int ldy, int polls);

/* ------------------------------------------------- device-pointer variants -- */
/* Hessian H = coeff_M M + coeff_K K(q) of the plan's element data into FP32
 * values_d (9*nnzb floats, the plan's CSR order), q_d = 3nV positions on the
 * device. values_d == NULL writes the plan's internal Hessian buffer (the one
 * bartels_plan_spmv_d and the Newton solver use). Enqueued on ctx's stream. */
int bartels_plan_hessian_d(bartels_ctx ctx, bartels_mesh_plan plan, int model, int psd_mode, double psd_tol,
                           int flags, double coeff_K, double coeff_M, const double *q_d, float *values_d);
/* y_d = H x_d (FP32, 3nV) with H in the plan's CSR order (values_d == NULL: the
 * plan's internal Hessian buffer). Rows of pinned vertices give 0. */
int bartels_plan_spmv_d(bartels_ctx ctx, bartels_mesh_plan plan, const float *values_d, const float *x_d,
                        float *y_d);
/* Implicit-Euler bookkeeping after a converged step in velocity form:
 * q_base += dt * v, x_hat = v (device v_d, 3nV). */
int bartels_newton_advance_implicit_euler_d(bartels_ctx ctx, bartels_mesh_plan plan, double dt, const double *v_d);

/* Device-pointer forms of bartels_tetmesh_q / bartels_tetmesh_dq
 * (linear_tetmesh_<model>_q / _dq, e.g. src/linear_tetmesh_neohookean_q.cpp:10-24,
 * src/linear_tetmesh_neohookean_dq.cpp:5-22) with the plan's element data (bartels_plan_set_element_data; for LINEAR_ELASTICITY
 * the stored params are the Lame pair): q_d 3nV device doubles; the energy goes
 * to the device scalar energy_d, the gradient to device g_d (3nV). Enqueued on
 * the context's stream without a host synchronisation, so no finiteness check
 * (the host forms return BARTELS_E_NONFINITE). Same kernels and summation
 * order as the host forms: identical results. */
int bartels_tetmesh_q_d(bartels_ctx ctx, bartels_mesh_plan plan, int model, const double *q_d, double *energy_d);
int bartels_tetmesh_dq_d(bartels_ctx ctx, bartels_mesh_plan plan, int model, const double *q_d, double *g_d);
/* Energy of every tet, psi(F) vol (linear_tet_{neohookean,stvk,corotational}_q
 * per element, src/linear_tet_neohookean_q.cpp:5-18, with the plan's element
 * data; for LINEAR_ELASTICITY the stored params are the Lame pair) at device
 * positions q_d into device e_d (nT doubles): the terms bartels_tetmesh_q_d
 * sums. FP64. */
int bartels_tetmesh_q_elements_d(bartels_ctx ctx, bartels_mesh_plan plan, int model, const double *q_d,
                                 double *e_d);

/* ------------------------------------------------- allocation-free variant -- */
/* Gradient of the elastic energy (as bartels_tetmesh_dq, with the plan's
 * element data) at device positions q_d (3nV doubles) into device g_d (3nV),
 * without allocating any memory: for callers that cannot call cudaMalloc,
 * such as a host application that reserves all device memory for its own
 * pool at start-up, a time-stepping loop that must not take cudaMalloc's
 * implicit device synchronisation, or a host that accounts every device
 * allocation. Its element-gradient scratch is a fixed array compiled into the
 * library (6 MiB, held by every GPU that loads it until the process exits),
 * so meshes of at most 65536 tets are accepted; larger ones return
 * BARTELS_E_UNSUPPORTED. The first call on a device looks up the array's
 * device address and keeps it for the life of the process (make that first
 * call before any stream capture; a device reset invalidates the address).
 * All calls share the array: calls that overlap on the GPU race.
 * This entry point has no counterpart in the reference. */
int bartels_tetmesh_dq_noalloc_d(bartels_ctx ctx, bartels_mesh_plan plan, int model, const double *q_d,
                                 double *g_d);

/* ------------------------------------------------------ 2D triangle meshes -- */
/* linear_tri2dmesh_* (src/linear_tri2dmesh_*.cpp): meshes in the plane, two DOFs
 * per vertex (q interleaved [x0 y0 x1 y1 ...]), E nT x 3 column-major 0-based,
 * dphidX nT x 6 (the column-major flatten of each 3x2 gradient matrix, as
 * linear_tri2dmesh_dphi_dX), area nT, params nT x 2 column-major (the tet
 * conventions: Neo-Hookean (C, D), StVK and corotational (lambda, mu), ARAP
 * column 0 = k, linear elasticity (Young's modulus, Poisson ratio)). The 2D
 * deformation gradient is embedded in 3D with F33 = 1, as the reference does.
 * The plan holds the CSR pattern (dim x dim vertex blocks; rows dim v .. dim v +
 * dim - 1 with the sorted columns of v's neighbours, as the reference's assemble); all
 * arithmetic is FP64 and every entry is summed over its triangles in triangle
 * order. */
typedef struct bartels_tri_plan_s *bartels_tri_plan;
/* dim: DOFs per vertex, 2 for the linear_tri2dmesh_* functions, 3 for
 * linear_tri3dmesh_* (triangles in space). */
int bartels_tri_plan_create(bartels_ctx ctx, int nV, int nT, const int *E, int dim, bartels_tri_plan *plan);
void bartels_tri_plan_destroy(bartels_tri_plan plan);
int bartels_tri_plan_csr_size(bartels_tri_plan plan, int *n, int64_t *nnz);
int bartels_tri_plan_csr_pattern(bartels_tri_plan plan, int *row_ptr, int *col_idx);
/* linear_tri2dmesh_dphi_dX (src/linear_tri2dmesh_dphi_dX.cpp:5-18,
 * src/linear_tri2d_dphi_dX.cpp:10-16); V nV x 2 column-major; area (optional)
 * = |det| / 2 of the edge matrix. */
int bartels_tri2dmesh_dphi_dX(bartels_ctx ctx, int nV, const double *V, int nT, const int *E, double *dphidX,
                              double *area);
/* Energy, gradient (2nV) and Hessian (CSR values in the plan's order) of model
 * (BARTELS_NEOHOOKEAN ... BARTELS_ARAP; the Hessian also takes
 * BARTELS_LINEAR_ELASTICITY, src/linear_tri2d_linear_elasticity_dq2.cpp:9-44).
 * psd_mode BARTELS_PSD_SIMPLE_FIX applies simple_psd_fix (src/simple_psd_fix.cpp:5-21)
 * to each 6x6 element matrix. */
int bartels_tri2dmesh_q(bartels_ctx ctx, bartels_tri_plan plan, int model, const double *q, const double *dphidX,
                        const double *area, const double *params, double *energy);
int bartels_tri2dmesh_dq(bartels_ctx ctx, bartels_tri_plan plan, int model, const double *q, const double *dphidX,
                         const double *area, const double *params, double *g);
int bartels_tri2dmesh_dq2(bartels_ctx ctx, bartels_tri_plan plan, int model, const double *q, const double *dphidX,
                          const double *area, const double *params, int psd_mode, double psd_tol,
                          double *csr_values);
/* linear_tri2dmesh_mass_matrix (src/linear_tri2dmesh_mass_matrix.cpp,
 * src/linear_tri2d_mass_matrix.cpp:10-32): density * area * (1/6, 1/12) x I2. */
int bartels_tri2dmesh_mass_matrix(bartels_ctx ctx, bartels_tri_plan plan, const double *density,
                                  const double *area, double *csr_values);
/* Named drop-ins: bartels_tri2dmesh_{neohookean,stvk,corotational,arap}_{q,dq,dq2}
 * (src/linear_tri2dmesh_<model>_{q,dq,dq2}.cpp) and
 * bartels_tri2dmesh_linear_elasticity_dq2. */
int bartels_tri2dmesh_neohookean_q(bartels_ctx ctx, bartels_tri_plan plan, const double *q, const double *dphidX,
                                   const double *area, const double *params, double *energy);
int bartels_tri2dmesh_neohookean_dq(bartels_ctx ctx, bartels_tri_plan plan, const double *q, const double *dphidX,
                                    const double *area, const double *params, double *g);
int bartels_tri2dmesh_neohookean_dq2(bartels_ctx ctx, bartels_tri_plan plan, const double *q, const double *dphidX,
                                     const double *area, const double *params, int psd_mode, double psd_tol,
                                     double *csr_values);
int bartels_tri2dmesh_stvk_q(bartels_ctx ctx, bartels_tri_plan plan, const double *q, const double *dphidX,
                             const double *area, const double *params, double *energy);
int bartels_tri2dmesh_stvk_dq(bartels_ctx ctx, bartels_tri_plan plan, const double *q, const double *dphidX,
                              const double *area, const double *params, double *g);
int bartels_tri2dmesh_stvk_dq2(bartels_ctx ctx, bartels_tri_plan plan, const double *q, const double *dphidX,
                               const double *area, const double *params, int psd_mode, double psd_tol,
                               double *csr_values);
int bartels_tri2dmesh_corotational_q(bartels_ctx ctx, bartels_tri_plan plan, const double *q, const double *dphidX,
                                     const double *area, const double *params, double *energy);
int bartels_tri2dmesh_corotational_dq(bartels_ctx ctx, bartels_tri_plan plan, const double *q, const double *dphidX,
                                      const double *area, const double *params, double *g);
int bartels_tri2dmesh_corotational_dq2(bartels_ctx ctx, bartels_tri_plan plan, const double *q, const double *dphidX,
                                       const double *area, const double *params, int psd_mode, double psd_tol,
                                       double *csr_values);
int bartels_tri2dmesh_arap_q(bartels_ctx ctx, bartels_tri_plan plan, const double *q, const double *dphidX,
                             const double *area, const double *params, double *energy);
int bartels_tri2dmesh_arap_dq(bartels_ctx ctx, bartels_tri_plan plan, const double *q, const double *dphidX,
                              const double *area, const double *params, double *g);
int bartels_tri2dmesh_arap_dq2(bartels_ctx ctx, bartels_tri_plan plan, const double *q, const double *dphidX,
                               const double *area, const double *params, int psd_mode, double psd_tol,
                               double *csr_values);
int bartels_tri2dmesh_linear_elasticity_dq2(bartels_ctx ctx, bartels_tri_plan plan, const double *q,
                                            const double *dphidX, const double *area, const double *params,
                                            int psd_mode, double psd_tol, double *csr_values);

/* ------------------------------------------------- triangles in space (3D) -- */
/* linear_tri3dmesh_dphi_dX (src/linear_tri3dmesh_dphi_dX.cpp,
 * src/linear_tri3d_dphi_dX.cpp:10-16): V nV x 3 column-major; dphidX nT x 9, the
 * column-major flatten of each 3x3 (rows 1, 2 = (T^T T)^-1 T^T, row 0 = minus
 * their sum); area (optional) = |e1 x e2| / 2. */
int bartels_tri3dmesh_dphi_dX(bartels_ctx ctx, int nV, const double *V, int nT, const int *E, double *dphidX,
                              double *area);
/* linear_tri3dmesh_stvk_dq2 (src/linear_tri3dmesh_stvk_dq2.cpp,
 * src/linear_tri3d_stvk_dq2.cpp:15-42): StVK membrane Hessian of a triangle mesh
 * in space, 3 DOFs per vertex (plan created with dim 3); per element the rest
 * normal N (nT x 3), the deformed normal n (nT x 3) and its derivative dndq
 * (nT x 27, the column-major flatten of dn/dqe 3x9), params (lambda, mu)
 * nT x 2; optional simple_psd_fix on each 9x9 element matrix. FP64. */
int bartels_tri3dmesh_stvk_dq2(bartels_ctx ctx, bartels_tri_plan plan, const double *q, const double *dphidX,
                               const double *N, const double *n, const double *dndq, const double *area,
                               const double *params, int psd_mode, double psd_tol, double *csr_values);

#ifdef __cplusplus
}
#endif
#endif /* BARTELS_GPU_H */
