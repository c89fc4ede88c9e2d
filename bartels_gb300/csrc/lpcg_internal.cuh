// Internal declarations of the learned preconditioner: the tensor-core GEMM,
// the factor pattern of a plan and the network object.
#pragma once

#include <cuda_bf16.h>

#include <cstdint>
#include <vector>

#include "internal.cuh"

namespace bartels {

// Y = act(X W^T + bias) (+ resid); X: M x K BF16 (row stride ldx), W: N x K BF16.
struct GemmArgs {
  int M = 0, N = 0, K = 0;
  const __nv_bfloat16 *x = nullptr;
  int ldx = 0;
  const __nv_bfloat16 *w = nullptr;
  const float *bias = nullptr;
  const float *resid = nullptr;
  int ldr = 0;
  int relu = 0;
  float *ypre = nullptr;  // X W^T + bias before the activation
  int ldp = 0;
  float *y = nullptr;
  int ldy = 0;
  __nv_bfloat16 *y2 = nullptr;
  int ldy2 = 0;
  int *err = nullptr;  // device int, set non-zero when a bounded wait gave up
  int probe_polls = 0;  // > 0: failure-path probe (no copy, no MMA; the first wait runs out)
};
int gemm_bf16(bartels_ctx ctx, const GemmArgs &g);

// Lower / upper block storage of a triangular factor on the plan's pattern.
//   lower row v: the blocks of columns j <= v (full-row positions 0 .. diag_pos[v]),
//                values in three scalar rows of 3 nl entries at 9 lrp[v];
//   upper row v: the blocks of columns j >= v (positions diag_pos[v] .. end),
//                values in three scalar rows of 3 nu entries at 9 urp[v].
//   low2up[l] : upper index (urp numbering) of lower block l transposed;
//   up2low[u] : lower index of upper block u transposed;
//   rev[p]    : full-pattern position of the reverse block of position p.
//   meta[v]   : {brp[v], lseg[v], useg[v], diag_pos[v] | row blocks << 16} for the PCG passes.
// The factor's BF16 values are kept per vertex as three scalar rows padded to a
// multiple of 4 entries (rsp = (3 n + 3) & ~3), starting at element lseg[v]
// (lower) or useg[v] (upper), so that a lane reads 4 values with one 8-byte load.
struct FactorPattern {
  int *lrp = nullptr, *urp = nullptr, *low2up = nullptr, *up2low = nullptr, *rev = nullptr;
  int4 *meta = nullptr;
  int64_t nnzl = 0, nnzu = 0;
  int64_t lsize = 0, usize = 0;  // padded BF16 elements of the lower / upper storage
  bool built = false;
  void release();
};
int plan_factor_pattern(bartels_mesh_plan plan, FactorPattern **out);

__host__ __device__ inline int padded_row(int nblocks) { return (3 * nblocks + 3) & ~3; }

// Factor G of the learned preconditioner for the plan's current Hessian values
// (FP32, scalar-CSR order): lower and upper storage, valid until the next call.
int lpcg_factor(bartels_lpcg net, bartels_mesh_plan plan, const float *values, const __nv_bfloat16 **gl,
                const __nv_bfloat16 **gu);

}  // namespace bartels

int lpcg_create(bartels_ctx ctx, bartels_lpcg *out);
void lpcg_destroy(bartels_lpcg n);
int lpcg_num_params();
int lpcg_set_params(bartels_lpcg n, const float *host);
int lpcg_get_params(bartels_lpcg n, float *host, float *grad_host);
int lpcg_train_step(bartels_lpcg n, bartels_mesh_plan plan, const float *values_d, const double *resid_d, int nrand,
                    unsigned seed, float lr, float clip, double *loss);
int lpcg_outputs(bartels_lpcg n, bartels_mesh_plan plan, const float *values_d, float *raw_host, float *gl_host);
bartels_ctx lpcg_ctx(bartels_lpcg n);
