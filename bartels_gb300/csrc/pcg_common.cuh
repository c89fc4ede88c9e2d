// Device helpers shared by the PCG loop (solver.cu) and the multigrid
// preconditioner (amg.cu): the device-side PCG state, deterministic block
// reductions, the block-row SpMV walk over the plan's value layout and the
// triangular-factor row walk.
#pragma once

#include <cuda_bf16.h>

#include <cstdint>

namespace bartels {

// Device-side PCG scalars. Reductions finish in the last block of the kernel
// that produces them (fixed summation order), so consumers read scalars.
struct PcgState {
  double rz;            // r.z of the current iterate
  double rr;            // r.r of the current iterate
  double pap;           // p.Ap of the current direction
  double rr0, tol2;
  float alpha, beta;    // step and direction coefficients, computed once by the last block
  int it;               // iterations completed in the current inner solve
  int done;
  int max_it;
  unsigned int count;   // blocks finished (last-block reductions)
  unsigned int loops;   // device-driven loop: body executions of the current inner solve
};

// 3x3 block-Jacobi apply: minv holds m00 m11 m22 m01 m02 m12 of each vertex's
// symmetric inverse diagonal block.
__device__ __forceinline__ void apply_minv(const float *__restrict__ minv, int v, const float *r, float *z) {
  const float *m = minv + 6ll * v;
  const float m00 = m[0], m11 = m[1], m22 = m[2], m01 = m[3], m02 = m[4], m12 = m[5];
  z[0] = m00 * r[0] + m01 * r[1] + m02 * r[2];
  z[1] = m01 * r[0] + m11 * r[1] + m12 * r[2];
  z[2] = m02 * r[0] + m12 * r[1] + m22 * r[2];
}

// Programmatic dependent launch: a kernel launched with programmatic stream
// serialisation (BT_LAUNCH_PDL) may be scheduled while its predecessor is
// finishing; pdl_wait() returns once the predecessor has completed and its
// memory is visible, so every such kernel calls it before touching any data
// (it returns at once for a kernel launched without the attribute).
// pdl_trigger() lets the successor be scheduled once every block of this
// kernel runs.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// ------------------------------------------------------------- reductions ---
__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_sumf(float v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// sum of blockDim-strided values of one double per thread; returns in thread 0
__device__ __forceinline__ double cta_sum(double v) {
  __shared__ double red[32];
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) red[w] = v;
  __syncthreads();
  double s = 0.0;
  if (w == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    s = lane < nw ? red[lane] : 0.0;
    s = warp_sum(s);
  }
  __syncthreads();
  return s;
}

// Last-block completion: returns true in every thread of the block that
// finished last (after all partials are visible).
__device__ __forceinline__ bool last_block(unsigned int *count) {
  __shared__ bool am_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned int prev = atomicAdd(count, 1u);
    am_last = (prev == gridDim.x - 1);
  }
  __syncthreads();
  return am_last;
}

// Block sum of per-thread FP32 partials: FP32 within a warp (fixed shuffle
// tree), FP64 across warps. Valid in thread 0. Keeps the FP64 pipe (1/64 of
// FP32 on GB300) off the per-element path.
__device__ __forceinline__ double cta_sum_f(float v) {
  __shared__ double redf[32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) redf[w] = (double)v;
  __syncthreads();
  double s = 0.0;
  if (w == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    s = lane < nw ? redf[lane] : 0.0;
    s = warp_sum(s);
  }
  __syncthreads();
  return s;
}

// deterministic sum of n partials (fixed order), valid in thread 0
__device__ __forceinline__ double sum_partials(const double *a, int n) {
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) acc += __ldcg(a + i);
  return cta_sum(acc);
}

// One vertex row of the block-layout SpMV, split in two so that no shuffle
// runs in a divergent region: spmv_row_acc (G lanes of a group walk the row's
// (block, component) pairs and read the three scalar rows at that column with
// streaming loads; xval(c) supplies the vector entry at scalar column c) runs
// only for an active group, group_reduce runs in every lane of the warp.
// ld_val: streaming load of one matrix value (FP32, or the BF16 copy the
// multigrid V-cycle uses on its finest level).
__device__ __forceinline__ float ld_val(const float *p) { return __ldcs(p); }
__device__ __forceinline__ float ld_val(const __nv_bfloat16 *p) { return __bfloat162float(__ldcs(p)); }

template <int G, class VT, class XV>
__device__ __forceinline__ void spmv_row_acc(int v, int sl, const int *__restrict__ brp, const int *__restrict__ bcol,
                                             const VT *__restrict__ val, XV &&xval, float &s0, float &s1,
                                             float &s2) {
  const int rb = __ldg(brp + v);
  const int rs = 3 * (__ldg(brp + v + 1) - rb);
  const VT *r0 = val + 9ll * rb;
  for (int e = sl; e < rs; e += G) {
    const int j = e / 3, l = e - 3 * j;
    const float xv = xval(3 * __ldg(bcol + rb + j) + l);
    s0 += ld_val(r0 + e) * xv;
    s1 += ld_val(r0 + rs + e) * xv;
    s2 += ld_val(r0 + 2 * rs + e) * xv;
  }
}

template <int G>
__device__ __forceinline__ void group_reduce(float &s0, float &s1, float &s2) {
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) {
    s0 += __shfl_xor_sync(0xffffffffu, s0, o);
    s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    s2 += __shfl_xor_sync(0xffffffffu, s2, o);
  }
}

// Warp-uniform walk over vertex rows: each warp takes 32/G consecutive rows
// per step, group g of the warp row vb + g (inactive past nV).
#define BT_ROW_LOOP_BEGIN(G)                                                      \
  const int lane_ = threadIdx.x & 31, sl = lane_ % (G), gw_ = lane_ / (G);       \
  const int warp_ = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;                \
  const int nwarps_ = (gridDim.x * blockDim.x) >> 5;                             \
  for (int vb_ = warp_ * (32 / (G)); vb_ < nV; vb_ += nwarps_ * (32 / (G))) {    \
    const int v = vb_ + gw_;                                                      \
    const bool active = v < nV;
#define BT_ROW_LOOP_END }

// ------------------------------------------- factor preconditioner (G^T G) ---
// z = G^T (G r) with G block-lower-triangular on the plan's pattern (the
// learned preconditioner). G is held twice: by rows of its lower part and by
// rows of G^T (the transposed blocks), so both products are row gathers.
//
// Row v of a triangular operand: blocks [b0, b0 + nblk) of the full pattern row
// (columns cols[j] = bcol[brp[v] + b0 + j]), BF16 values in three scalar rows of
// rs = 3 nblk entries padded to rsp (a multiple of 4). Each lane takes 4
// consecutive columns per step: one 8-byte load per scalar row, and the 4
// vector entries of the (at most two) blocks those columns fall in.
// meta[v] = {brp, lower segment, upper segment, diag | nblocks << 16}.
template <int G, class XV>
__device__ __forceinline__ void tri_row_acc4(int sl, const int *__restrict__ cols, const __nv_bfloat16 *__restrict__ r0,
                                             int rs, int rsp, XV &&xval, float &s0, float &s1, float &s2) {
  for (int e0 = 4 * sl; e0 < rs; e0 += 4 * G) {
    const uint2 w0 = __ldcs(reinterpret_cast<const uint2 *>(r0 + e0));
    const uint2 w1 = __ldcs(reinterpret_cast<const uint2 *>(r0 + rsp + e0));
    const uint2 w2 = __ldcs(reinterpret_cast<const uint2 *>(r0 + 2 * rsp + e0));
    const int j0 = e0 / 3, l0 = e0 - 3 * j0;
    const int c0 = __ldg(cols + j0);
    const int c1 = 3 * (j0 + 1) < rs ? __ldg(cols + j0 + 1) : 0;
    float xv[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int l = l0 + q;
      const int c = l >= 3 ? c1 : c0;
      xv[q] = e0 + q < rs ? xval(3 * c + (l >= 3 ? l - 3 : l)) : 0.f;
    }
    const uint32_t u0[2] = {w0.x, w0.y}, u1[2] = {w1.x, w1.y}, u2[2] = {w2.x, w2.y};
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      s0 += __uint_as_float(u0[h] << 16) * xv[2 * h] + __uint_as_float(u0[h] & 0xFFFF0000u) * xv[2 * h + 1];
      s1 += __uint_as_float(u1[h] << 16) * xv[2 * h] + __uint_as_float(u1[h] & 0xFFFF0000u) * xv[2 * h + 1];
      s2 += __uint_as_float(u2[h] << 16) * xv[2 * h] + __uint_as_float(u2[h] & 0xFFFF0000u) * xv[2 * h + 1];
    }
  }
}

// Row v of the padded FP32 copy of the values (three scalar rows of rs
// entries, each padded with zeros to rsp, a multiple of 4): each lane takes 4
// consecutive columns per step with one 16-byte load per scalar row.
template <int G, class XV>
__device__ __forceinline__ void row_acc4f(int sl, const int *__restrict__ cols, const float *__restrict__ r0, int rs,
                                          int rsp, XV &&xval, float &s0, float &s1, float &s2) {
  for (int e0 = 4 * sl; e0 < rs; e0 += 4 * G) {
    const float4 w0 = __ldcs(reinterpret_cast<const float4 *>(r0 + e0));
    const float4 w1 = __ldcs(reinterpret_cast<const float4 *>(r0 + rsp + e0));
    const float4 w2 = __ldcs(reinterpret_cast<const float4 *>(r0 + 2 * rsp + e0));
    const int j0 = e0 / 3, l0 = e0 - 3 * j0;
    const int c0 = __ldg(cols + j0);
    const int c1 = 3 * (j0 + 1) < rs ? __ldg(cols + j0 + 1) : 0;
    float xv[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int l = l0 + q;
      const int c = l >= 3 ? c1 : c0;
      xv[q] = e0 + q < rs ? xval(3 * c + (l >= 3 ? l - 3 : l)) : 0.f;
    }
    s0 += w0.x * xv[0] + w0.y * xv[1] + w0.z * xv[2] + w0.w * xv[3];
    s1 += w1.x * xv[0] + w1.y * xv[1] + w1.z * xv[2] + w1.w * xv[3];
    s2 += w2.x * xv[0] + w2.y * xv[1] + w2.z * xv[2] + w2.w * xv[3];
  }
}

}  // namespace bartels
