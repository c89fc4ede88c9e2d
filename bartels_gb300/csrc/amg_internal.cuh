// Internal declarations of the aggregation multigrid preconditioner (amg.cu).
#pragma once

#include <cuda_bf16.h>

#include <cstdint>
#include <vector>

#include "internal.cuh"

namespace bartels {

struct FactorPattern;
struct PcgState;

// One level of the hierarchy. Level 0 is the plan's Hessian (3x3 blocks in the
// plan's value layout, pinned vertices excluded); coarse levels hold 6x6 blocks
// (3 translations + 3 rotations per aggregate), row-major, in block-CSR order.
struct MgLevel {
  int n = 0;       // nodes (level 0: the plan's vertices)
  int bs = 0;      // DOFs per node: 3 on level 0, 6 on coarse levels
  int64_t nnzb = 0;
  int *rp = nullptr, *ci = nullptr, *dpos = nullptr;  // coarse levels: block pattern, diagonal positions
  float *val = nullptr;                               // coarse levels: 36 floats per block
  // coarse levels: BF16 copy (A + A^T) / 2 of val, exactly symmetric, read by
  // the smoothing, residual and power-iteration kernels; rev = position of
  // the transposed block
  __nv_bfloat16 *val16 = nullptr;
  int *rev = nullptr;
  float *dinv = nullptr;                              // coarse levels: 36 floats per node (inverse diagonal block)
  // transfer to the next coarser level (none on the coarsest)
  int nc = 0;                         // nodes of the next level
  int *agg = nullptr;                 // n: aggregate of each node, -1 outside the system (pinned)
  int *mptr = nullptr, *midx = nullptr;  // members of each aggregate, ascending
  float *Q = nullptr;                 // n x bs x 6 (row-major): the tentative prolongator block of each node
  int *gptr = nullptr;                // next level's nnzb + 1: Galerkin contributions per coarse block
  int2 *gent = nullptr;               // (fine row, fine block index) of each contribution, in summation order
  // work vectors (bs * n floats)
  float *b = nullptr, *x = nullptr, *x2 = nullptr, *r = nullptr, *d = nullptr, *d2 = nullptr;
  int deg = 1;  // Chebyshev degree of the smoother on this level
};

constexpr int kMgMaxLevels = 12;
constexpr int kMgCoef = 16;  // per level: 1/theta, then (c1, c2) per further Chebyshev step

struct MgHierarchy {
  std::vector<MgLevel> lv;
  int dense = 0;          // the coarsest level is solved with its dense inverse
  int nd = 0;             // dense size (6 x nodes of the coarsest level)
  int coarse_blockdiag = 0;  // coarsest level is block diagonal: its block-Jacobi solve is exact
  float *ainv = nullptr;  // nd x nd
  float *coef = nullptr;  // kMgMaxLevels x kMgCoef Chebyshev coefficients (device)
  double *norms = nullptr;  // 2 per level: squared norms of the last two power iterates
  double *part = nullptr;   // reduction partials
  int nparts = 0;
  int pinned_gen = -1;    // plan->pinned_gen the hierarchy was built for
  int64_t coarse_nnz = 0; // stored entries of all coarse levels (operator complexity)
  PcgState *st_once = nullptr;  // state for a single application outside PCG
  double *segn = nullptr;       // per-segment norms of the finest level's last two power iterates
  int segn_n = 0;
  // BF16 copy of the finest level's values, made exactly symmetric, for the
  // V-cycle's own SpMVs (nullptr: the FP32 values are used). Vertex v's three
  // scalar rows start at a16_off[v] and are each padded with zeros to
  // padded_row(nb) entries (a multiple of 4), so a lane reads 4 values with
  // one 8-byte load.
  __nv_bfloat16 *a16 = nullptr;
  int *a16_off = nullptr;
  std::vector<void *> allocs;
  ~MgHierarchy();
};

// Smoother of level 0: block-Jacobi (minv, 6 floats per vertex) or the learned
// factor M = G^T G (gl / gu in the factor pattern fp).
struct MgSmoother {
  const float *minv = nullptr;
  const __nv_bfloat16 *gl = nullptr, *gu = nullptr;
  const FactorPattern *fp = nullptr;
};

// Build (or keep) the hierarchy for the plan's pattern and pinned set.
int mg_prepare(bartels_ctx ctx, bartels_mesh_plan plan);
void mg_destroy(MgHierarchy *mg);
// Galerkin products, inverse diagonal blocks, the coarsest inverse and the
// smoothers' eigenvalue bounds for the Hessian values (plan layout).
int mg_setup_numeric(bartels_ctx ctx, bartels_mesh_plan plan, const float *values, const MgSmoother &sm);
// z = B r (one V-cycle) for the PCG loop: every kernel is a no-op once st->done;
// the last one also forms r.z, beta = r.z / r.z_old and stores r.z in st.
// pre_done: the level-0 pre-smoothing was taken by mg_enqueue_update (block-
// Jacobi smoother only).
int mg_enqueue_apply(bartels_ctx ctx, bartels_mesh_plan plan, const float *values, const MgSmoother &sm,
                     const float *r, float *z, float *y, double *part, PcgState *st, bool pre_done);
// The PCG update (x += alpha p, r -= alpha Ap, r.r, iteration count and
// convergence test) fused with the level-0 block-Jacobi pre-smoothing of the
// next V-cycle.
int mg_enqueue_update(bartels_ctx ctx, bartels_mesh_plan plan, const MgSmoother &sm, const float *pa,
                      const float *pb, const float *ap, float *x, float *r, double *part, PcgState *st);
// z = B r once (no PCG state), for tests of the preconditioner itself.
int mg_apply_once(bartels_ctx ctx, bartels_mesh_plan plan, const float *values, const MgSmoother &sm, const float *r,
                  float *z);

}  // namespace bartels
