// Linear solve and Newton driver.
//
// PCG: FP32 SpMV / vectors with a 3x3 block-Jacobi preconditioner, captured as
// CUDA graphs of a fixed number of iterations that become no-ops once the
// device-side convergence flag is set. An outer FP64 loop recomputes the true
// residual b - A x in FP64 and restarts PCG on it (iterative refinement) until
// ||b - A x|| <= rel_tol ||b||.
//
// Newton: gradient (FP64) -> Hessian (FP32, fused assembly) -> PCG -> the
// reference's backtracking line search (src/linesearch_backtracking_bisection.cpp:17-30)
// on the device-evaluated FP64 objective, following newtons_method_bisection
// (include/optimization_gradient_based.h:77-106).
#include <nvtx3/nvToolsExt.h>

#include <chrono>
#include <climits>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <vector>

#include "devmath.cuh"
#include "internal.cuh"
#include "amg_internal.cuh"
#include "lpcg_internal.cuh"
#include "pcg_common.cuh"

namespace bartels {

int launch_prep_u(bartels_ctx ctx, bartels_mesh_plan plan, const double *x, const double *q_base, double scale,
                  bool displacement, float4 *u);
int launch_hess(bartels_ctx ctx, bartels_mesh_plan plan, int model, int psd_mode, const float4 *u, int add_identity,
                float cK, float cM, float tol, int flags, float *values);

constexpr int kVecBlocksPerSM = 8;
constexpr int kSpmvBlocksPerSM = 8;

// ------------------------------------------------------------------ SpMV ---
// refinement residual r = b - A x of a generic scalar CSR (the drop-in search
// direction): FP64 products (with the exact FP64 values when given), one warp
// per row, rounded to the FP32 residual the inner solve takes; partial sums of r.r
__global__ void __launch_bounds__(256)
k_resid_csr64(int n, const int *__restrict__ rp, const int *__restrict__ ci, const float *__restrict__ val,
              const double *__restrict__ val64, const double *__restrict__ x, const double *__restrict__ b,
              float *__restrict__ r, double *__restrict__ partial) {
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  double acc = 0.0;
  for (int i = warp; i < n; i += nwarps) {
    double s = 0.0;
    for (int k = rp[i] + lane; k < rp[i + 1]; k += 32) s += (val64 ? val64[k] : (double)val[k]) * x[ci[k]];
    s = warp_sum(s);
    if (lane == 0) {
      double q = b[i] - s;
      r[i] = (float)q;
      acc += q * q;
    }
  }
  double s = cta_sum(acc);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

// ------------------------------------------------------- block Jacobi ------
// inverse of each 3x3 diagonal block (FP64 inversion, FP32 storage). Blocks
// that are pinned get 0; singular or indefinite blocks fall back to the
// inverse diagonal.
// 6 floats per block: m00 m11 m22 m01 m02 m12 of the symmetric inverse
__device__ void store_inv3(const double *A0, float *out) {
  double A[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) A[i + 3 * j] = 0.5 * (A0[i + 3 * j] + A0[j + 3 * i]);
  double G[9];
  cof3(G, A);
  double det = A[0] * G[0] + A[1] * G[1] + A[2] * G[2];
  if (det > 0.0 && isfinite(det)) {
    out[0] = (float)(G[0] / det);
    out[1] = (float)(G[4] / det);
    out[2] = (float)(G[8] / det);
    out[3] = (float)(G[3] / det);
    out[4] = (float)(G[6] / det);
    out[5] = (float)(G[7] / det);
  } else {
    for (int i = 0; i < 3; ++i) {
      double d = A[i + 3 * i];
      out[i] = (d != 0.0 && isfinite(d)) ? (float)(1.0 / d) : 1.f;
    }
    out[3] = out[4] = out[5] = 0.f;
  }
}

__global__ void k_minv_blk(int nV, const int *__restrict__ brp, const int *__restrict__ diag_pos,
                           const float *__restrict__ val, const unsigned char *__restrict__ pinned,
                           float *__restrict__ minv) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nV; v += gridDim.x * blockDim.x) {
    const int rb = brp[v], rs = 3 * (brp[v + 1] - rb), j = diag_pos[v];
    const float *r0 = val + 9ll * rb;
    double A[9];
    for (int k = 0; k < 3; ++k)
      for (int l = 0; l < 3; ++l) A[k + 3 * l] = r0[k * rs + 3 * j + l];
    float out[6];
    if (pinned && pinned[v]) {
      for (int i = 0; i < 6; ++i) out[i] = 0.f;
    } else {
      store_inv3(A, out);
    }
    for (int i = 0; i < 6; ++i) minv[6ll * v + i] = out[i];
  }
}

__global__ void k_minv_csr(int nb, int n, const int *__restrict__ rp, const int *__restrict__ ci,
                           const float *__restrict__ val, float *__restrict__ minv) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nb; v += gridDim.x * blockDim.x) {
    double A[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int k = 0; k < 3; ++k) {
      const int row = 3 * v + k;
      if (row >= n) {
        A[k + 3 * k] = 1.0;
        continue;
      }
      for (int e = rp[row]; e < rp[row + 1]; ++e) {
        const int c = ci[e] - 3 * v;
        if (c >= 0 && c < 3) A[k + 3 * c] += val[e];
      }
    }
    float out[6];
    store_inv3(A, out);
    for (int i = 0; i < 6; ++i) minv[6ll * v + i] = out[i];
  }
}


// start of an inner solve: x = 0, r = rres (the refinement residual), z = M^-1 r. A fresh solve
// (cont = 0) clears p and the iteration count; a continued one (cont = 1, the
// reliable update) keeps the previous pass's last direction and iteration
// count, and takes beta = r'.z' / r_k.z_k against the replaced residual r'
// (r_k.z_k = r.z / beta of the previous pass's last update).
__global__ void k_pcg_init(int nb, int n, const float *__restrict__ rres, const float *__restrict__ minv,
                           float *__restrict__ x, float *__restrict__ r, float *__restrict__ z,
                           float *__restrict__ p0, float *__restrict__ p1, double *__restrict__ part_a,
                           double *__restrict__ part_b, PcgState *__restrict__ st, double inner_rel2, double abs_tol2,
                           int max_it, int cont) {
  pdl_wait();
  pdl_trigger();
  float arz = 0.f, arr = 0.f;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nb; v += gridDim.x * blockDim.x) {
    float rv[3], zv[3];
    for (int k = 0; k < 3; ++k) rv[k] = (3 * v + k < n) ? rres[3 * v + k] : 0.f;
    apply_minv(minv, v, rv, zv);
    for (int k = 0; k < 3; ++k) {
      const int i = 3 * v + k;
      if (i < n) {
        x[i] = 0.f;
        r[i] = rv[k];
        z[i] = zv[k];
        if (!cont) {
          p0[i] = 0.f;
          p1[i] = 0.f;
        }
        arz += rv[k] * zv[k];
        arr += rv[k] * rv[k];
      }
    }
  }
  double s = cta_sum_f(arz);
  if (threadIdx.x == 0) part_a[blockIdx.x] = s;
  s = cta_sum_f(arr);
  if (threadIdx.x == 0) part_b[blockIdx.x] = s;
  if (last_block(&st->count)) {
    const double rz = sum_partials(part_a, gridDim.x);
    const double rr = sum_partials(part_b, gridDim.x);
    if (threadIdx.x == 0) {
      const double rz_old = (cont && st->beta > 0.f) ? st->rz / (double)st->beta : 0.0;
      st->beta = (rz_old > 0.0 && rz_old < HUGE_VAL) ? (float)(rz / rz_old) : 0.f;
      st->rz = rz;
      st->rr = rr;
      st->rr0 = rr;
      st->pap = 0.0;
      st->alpha = 0.f;
      st->tol2 = fmax(inner_rel2 * rr, abs_tol2);
      if (!cont) st->it = 0;
      st->loops = 0;
      st->max_it = st->it + max_it;
      st->done = (rr <= st->tol2 || max_it <= 0 || !(rr == rr)) ? 1 : 0;
      st->count = 0;
    }
  }
}

// y = A x with the PCG's row mapping (rows of pinned vertices give 0)
template <int G>
__global__ void __launch_bounds__(256)
k_spmv_blk_g(int nV, const int *__restrict__ brp, const int *__restrict__ bcol, const float *__restrict__ val,
             const float *__restrict__ x, float *__restrict__ y, const unsigned char *__restrict__ pinned) {
  BT_ROW_LOOP_BEGIN(G)
  float s0 = 0.f, s1 = 0.f, s2 = 0.f;
  if (active) spmv_row_acc<G>(v, sl, brp, bcol, val, [&](int c) { return __ldg(x + c); }, s0, s1, s2);
  group_reduce<G>(s0, s1, s2);
  if (active && sl == 0) {
    if (pinned && pinned[v]) s0 = s1 = s2 = 0.f;
    y[3 * v] = s0;
    y[3 * v + 1] = s1;
    y[3 * v + 2] = s2;
  }
  BT_ROW_LOOP_END
}

// Direction p = z + beta p_old (into the other p buffer), 4 vertices = 12
// floats = 3 aligned float4 per thread, scalar tail.
__global__ void __launch_bounds__(256)
k_pcg_dir(int n, const float *__restrict__ z, float *__restrict__ pa, float *__restrict__ pb,
          const PcgState *__restrict__ st) {
  pdl_wait();
  pdl_trigger();
  if (st->done) return;
  const int it = st->it;
  const float beta = st->beta;
  const float *p_old = (it & 1) ? pa : pb;
  float *p_new = (it & 1) ? pb : pa;
  const int n4 = n / 4;
  const float4 *z4 = reinterpret_cast<const float4 *>(z);
  const float4 *o4 = reinterpret_cast<const float4 *>(p_old);
  float4 *n4p = reinterpret_cast<float4 *>(p_new);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += gridDim.x * blockDim.x) {
    const float4 a = __ldcg(z4 + i), o = __ldcg(o4 + i);
    n4p[i] = make_float4(a.x + beta * o.x, a.y + beta * o.y, a.z + beta * o.z, a.w + beta * o.w);
  }
  for (int i = 4 * n4 + blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    p_new[i] = z[i] + beta * p_old[i];
}

// ap = A p (block layout), partials of p.Ap; alpha in the last block. PAD:
// val is the padded copy of the values (rows at off[v], 4 per 16-byte load),
// otherwise the plan's own layout.
template <int G, bool PAD>
__global__ void __launch_bounds__(256)
k_pcg_spmv_blk(int nV, const int *__restrict__ brp, const int *__restrict__ bcol, const float *__restrict__ val,
               const int *__restrict__ off, const float *__restrict__ pa, const float *__restrict__ pb,
               float *__restrict__ ap, const unsigned char *__restrict__ pinned, double *__restrict__ part,
               PcgState *__restrict__ st) {
  pdl_wait();
  pdl_trigger();
  if (st->done) return;
  const float *p = (st->it & 1) ? pb : pa;
  float acc = 0.f;
  BT_ROW_LOOP_BEGIN(G)
  float s0 = 0.f, s1 = 0.f, s2 = 0.f;
  if (active) {
    if constexpr (PAD) {
      const int rb = __ldg(brp + v), nb = __ldg(brp + v + 1) - rb;
      row_acc4f<G>(sl, bcol + rb, val + __ldg(off + v), 3 * nb, padded_row(nb), [&](int c) { return __ldcg(p + c); },
                   s0, s1, s2);
    } else {
      spmv_row_acc<G>(v, sl, brp, bcol, val, [&](int c) { return __ldcg(p + c); }, s0, s1, s2);
    }
  }
  group_reduce<G>(s0, s1, s2);
  if (active && sl == 0) {
    if (pinned && pinned[v]) s0 = s1 = s2 = 0.f;
    ap[3 * v] = s0;
    ap[3 * v + 1] = s1;
    ap[3 * v + 2] = s2;
    acc += __ldcg(p + 3 * v) * s0 + __ldcg(p + 3 * v + 1) * s1 + __ldcg(p + 3 * v + 2) * s2;
  }
  BT_ROW_LOOP_END
  double s = cta_sum_f(acc);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
  if (last_block(&st->count)) {
    const double pap = sum_partials(part, gridDim.x);
    if (threadIdx.x == 0) {
      st->pap = pap;
      st->alpha = (float)(st->rz / pap);
      st->count = 0;
    }
  }
}

// Copy of the values into the padded layout (warp per vertex row); the pads
// are zeroed when the buffer is allocated and never written.
__global__ void __launch_bounds__(256)
k_pad_values(int nV, const int *__restrict__ brp, const int *__restrict__ off, const float *__restrict__ val,
             float *__restrict__ vpad) {
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int v = warp; v < nV; v += nwarps) {
    const int rb = brp[v], nb = brp[v + 1] - rb, rs = 3 * nb, rsp = padded_row(nb);
    const float *src = val + 9ll * rb;
    float *dst = vpad + off[v];
#pragma unroll
    for (int k = 0; k < 3; ++k)
      for (int e = lane; e < rs; e += 32) dst[k * rsp + e] = __ldcs(src + k * rs + e);
  }
}

// ap = A p for a generic scalar CSR (one warp per row), partials of p.Ap.
__global__ void __launch_bounds__(256)
k_pcg_spmv_csr(int n, const int *__restrict__ rp, const int *__restrict__ ci, const float *__restrict__ val,
               const float *__restrict__ pa, const float *__restrict__ pb, float *__restrict__ ap,
               double *__restrict__ part, PcgState *__restrict__ st) {
  pdl_wait();
  pdl_trigger();
  if (st->done) return;
  const float *p = (st->it & 1) ? pb : pa;
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  float acc = 0.f;
  for (int i = warp; i < n; i += nwarps) {
    float s = 0.f;
    for (int k = rp[i] + lane; k < rp[i + 1]; k += 32) s += val[k] * __ldcg(p + ci[k]);
    s = warp_sumf(s);
    if (lane == 0) {
      ap[i] = s;
      acc += __ldcg(p + i) * s;
    }
  }
  double s = cta_sum_f(acc);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
  if (last_block(&st->count)) {
    const double pap = sum_partials(part, gridDim.x);
    if (threadIdx.x == 0) {
      st->pap = pap;
      st->alpha = (float)(st->rz / pap);
      st->count = 0;
    }
  }
}

// alpha = rz / pAp; x += alpha p; r -= alpha Ap; z = M^-1 r; r.z and r.r;
// convergence test, beta and iteration count in the last block. One thread
// per group of 4 vertices (12 floats = 3 aligned float4 per vector, 24 floats
// = 6 float4 of block-Jacobi); the ragged tail is handled per vertex.
__device__ __forceinline__ void update_vertex(int v, float alpha, const float *__restrict__ minv,
                                              const float *__restrict__ p, const float *__restrict__ ap,
                                              float *__restrict__ x, float *__restrict__ r, float *__restrict__ z,
                                              float &arz, float &arr) {
  float rv[3], zv[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int i = 3 * v + k;
    x[i] += alpha * __ldcg(p + i);
    rv[k] = r[i] - alpha * __ldcg(ap + i);
    r[i] = rv[k];
  }
  apply_minv(minv, v, rv, zv);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    z[3 * v + k] = zv[k];
    arz += rv[k] * zv[k];
    arr += rv[k] * rv[k];
  }
}

__global__ void __launch_bounds__(256)
k_pcg_update(int nb, int n, const float *__restrict__ minv, const float *__restrict__ pa,
             const float *__restrict__ pb, const float *__restrict__ ap, float *__restrict__ x,
             float *__restrict__ r, float *__restrict__ z, double *__restrict__ part_a, double *__restrict__ part_b,
             PcgState *__restrict__ st) {
  pdl_wait();
  pdl_trigger();
  if (st->done) return;
  const int it = st->it;
  const float *p = (it & 1) ? pb : pa;
  const float alpha = st->alpha;
  float arz = 0.f, arr = 0.f;
  const int nfull = (n % 3 == 0) ? nb / 4 : 0;  // groups of 4 complete vertices (vector path)
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < nfull; g += gridDim.x * blockDim.x) {
    const float4 *p4 = reinterpret_cast<const float4 *>(p) + 3 * g;
    const float4 *a4 = reinterpret_cast<const float4 *>(ap) + 3 * g;
    float4 *x4 = reinterpret_cast<float4 *>(x) + 3 * g;
    float4 *r4 = reinterpret_cast<float4 *>(r) + 3 * g;
    float4 *z4 = reinterpret_cast<float4 *>(z) + 3 * g;
    const float4 *m4 = reinterpret_cast<const float4 *>(minv) + 6 * g;
    float pv[12], av[12], xv[12], rv[12], mv[24], zv[12];
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      const float4 a = __ldcg(p4 + q), b = __ldcg(a4 + q), c = x4[q], d = r4[q];
      pv[4 * q] = a.x; pv[4 * q + 1] = a.y; pv[4 * q + 2] = a.z; pv[4 * q + 3] = a.w;
      av[4 * q] = b.x; av[4 * q + 1] = b.y; av[4 * q + 2] = b.z; av[4 * q + 3] = b.w;
      xv[4 * q] = c.x; xv[4 * q + 1] = c.y; xv[4 * q + 2] = c.z; xv[4 * q + 3] = c.w;
      rv[4 * q] = d.x; rv[4 * q + 1] = d.y; rv[4 * q + 2] = d.z; rv[4 * q + 3] = d.w;
    }
#pragma unroll
    for (int q = 0; q < 6; ++q) {
      const float4 m = __ldg(m4 + q);
      mv[4 * q] = m.x; mv[4 * q + 1] = m.y; mv[4 * q + 2] = m.z; mv[4 * q + 3] = m.w;
    }
#pragma unroll
    for (int i = 0; i < 12; ++i) {
      xv[i] += alpha * pv[i];
      rv[i] -= alpha * av[i];
    }
#pragma unroll
    for (int w = 0; w < 4; ++w) {
      const float *m = mv + 6 * w;
      const float *rr = rv + 3 * w;
      zv[3 * w] = m[0] * rr[0] + m[3] * rr[1] + m[4] * rr[2];
      zv[3 * w + 1] = m[3] * rr[0] + m[1] * rr[1] + m[5] * rr[2];
      zv[3 * w + 2] = m[4] * rr[0] + m[5] * rr[1] + m[2] * rr[2];
    }
#pragma unroll
    for (int i = 0; i < 12; ++i) {
      arz += rv[i] * zv[i];
      arr += rv[i] * rv[i];
    }
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      x4[q] = make_float4(xv[4 * q], xv[4 * q + 1], xv[4 * q + 2], xv[4 * q + 3]);
      r4[q] = make_float4(rv[4 * q], rv[4 * q + 1], rv[4 * q + 2], rv[4 * q + 3]);
      z4[q] = make_float4(zv[4 * q], zv[4 * q + 1], zv[4 * q + 2], zv[4 * q + 3]);
    }
  }
  // tail (and the scalar path when n is not 3 nb)
  for (int v = 4 * nfull + blockIdx.x * blockDim.x + threadIdx.x; v < nb; v += gridDim.x * blockDim.x) {
    if (3 * v + 2 < n) {
      update_vertex(v, alpha, minv, p, ap, x, r, z, arz, arr);
    } else {
      float rv[3] = {0.f, 0.f, 0.f}, zv[3];
      for (int k = 0; k < 3; ++k)
        if (3 * v + k < n) {
          x[3 * v + k] += alpha * p[3 * v + k];
          rv[k] = r[3 * v + k] - alpha * ap[3 * v + k];
          r[3 * v + k] = rv[k];
        }
      apply_minv(minv, v, rv, zv);
      for (int k = 0; k < 3; ++k)
        if (3 * v + k < n) {
          z[3 * v + k] = zv[k];
          arz += rv[k] * zv[k];
          arr += rv[k] * rv[k];
        }
    }
  }
  double s = cta_sum_f(arz);
  if (threadIdx.x == 0) part_a[blockIdx.x] = s;
  s = cta_sum_f(arr);
  if (threadIdx.x == 0) part_b[blockIdx.x] = s;
  if (last_block(&st->count)) {
    const double rz = sum_partials(part_a, gridDim.x);
    const double rr = sum_partials(part_b, gridDim.x);
    if (threadIdx.x == 0) {
      st->beta = (float)(rz / st->rz);
      st->rz = rz;
      st->rr = rr;
      st->it = it + 1;
      if (rr <= st->tol2 || it + 1 >= st->max_it || !(rr == rr)) st->done = 1;
      st->count = 0;
    }
  }
}

// x += dx (FP64) and x split into two floats, x = xh + xl to ~2^-48 relative
// (the vector the refinement residual gathers).
__global__ void k_axpy64(int n, const float *__restrict__ dx, double *__restrict__ x, float *__restrict__ xh,
                         float *__restrict__ xl) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double v = dx ? x[i] + (double)dx[i] : x[i];
    if (dx) x[i] = v;
    const float h = (float)v;
    xh[i] = h;
    xl[i] = (float)(v - (double)h);
  }
}

// b split into two floats, b = bh + bl to ~2^-48 relative (once per solve)
__global__ void k_split64(int n, const double *__restrict__ b, float *__restrict__ bh, float *__restrict__ bl) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double v = b[i];
    const float h = (float)v;
    bh[i] = h;
    bl[i] = (float)(v - (double)h);
  }
}

// ---------------------------------------------- float-float residual -------
// GB300 runs FP64 at a small fraction of its FP32 rate, so the refinement
// residual r = b - A x works in float-float arithmetic (Dekker / Knuth
// error-free transformations): each product v (xh + xl) is v xh exactly as
// p + pe (pe by FMA) plus v xl, and the sums carry their rounding errors in a
// second float (TwoSum). The explicit-rounding intrinsics keep the compiler
// from fusing the additions into FMAs, which would break the transformations.
// The relative error of a row sum is ~2^-48 of sum |A_ij x_j|; FP64 is used
// only once per row (b - s and r.r).
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ void ff_mac(float v, float xh, float xl, float &h, float &l) {
  const float p = __fmul_rn(v, xh);
  const float pe = __fmaf_rn(v, xh, -p);
  float t, e;
  two_sum(h, p, t, e);
  h = t;
  l = __fadd_rn(l, __fadd_rn(e, __fmaf_rn(v, xl, pe)));
}

template <int G>
__device__ __forceinline__ void ff_group_reduce(float &h, float &l) {
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) {
    const float h2 = __shfl_xor_sync(0xffffffffu, h, o), l2 = __shfl_xor_sync(0xffffffffu, l, o);
    float t, e;
    two_sum(h, h2, t, e);
    h = t;
    l = __fadd_rn(__fadd_rn(l, l2), e);
  }
}

// r = b - A x (block layout, x = xh + xl, b = bh + bl), rounded to FP32 (the
// inner solve's residual); partial sums of r.r per block. No FP64 work: on
// this GPU one FP64 warp instruction costs about as much as 64 FP32 ones.
template <int G>
__global__ void __launch_bounds__(256)
k_resid_blk_ff(int nV, const int *__restrict__ brp, const int *__restrict__ bcol, const float *__restrict__ val,
               const float *__restrict__ xh, const float *__restrict__ xl, const float *__restrict__ bh,
               const float *__restrict__ bl, float *__restrict__ r, const unsigned char *__restrict__ pinned,
               double *__restrict__ partial) {
  float acc = 0.f;
  BT_ROW_LOOP_BEGIN(G)
  float h[3] = {0.f, 0.f, 0.f}, l[3] = {0.f, 0.f, 0.f};
  if (active) {
    const int rb = __ldg(brp + v);
    const int rs = 3 * (__ldg(brp + v + 1) - rb);
    const float *r0 = val + 9ll * rb;
    for (int e = sl; e < rs; e += G) {
      const int j = e / 3, c = 3 * __ldg(bcol + rb + j) + (e - 3 * j);
      const float a = __ldg(xh + c), al = __ldg(xl + c);
      ff_mac(__ldcs(r0 + e), a, al, h[0], l[0]);
      ff_mac(__ldcs(r0 + rs + e), a, al, h[1], l[1]);
      ff_mac(__ldcs(r0 + 2 * rs + e), a, al, h[2], l[2]);
    }
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) ff_group_reduce<G>(h[k], l[k]);
  if (active && sl == 0) {
    const bool pin = pinned && pinned[v];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      // (bh + bl) - (h + l) in float-float, rounded once
      float t, e;
      two_sum(__ldg(bh + 3 * v + k), -h[k], t, e);
      const float q = pin ? 0.f : __fadd_rn(t, __fadd_rn(e, __fsub_rn(__ldg(bl + 3 * v + k), l[k])));
      r[3 * v + k] = q;
      acc += q * q;
    }
  }
  BT_ROW_LOOP_END
  double s = cta_sum_f(acc);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

__global__ void k_scale_copy(int n, double a, const double *__restrict__ x, double *__restrict__ y) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) y[i] = a * x[i];
}

__global__ void k_axpy_to(int n, const double *__restrict__ x, double a, const double *__restrict__ d,
                          double *__restrict__ y) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) y[i] = x[i] + a * d[i];
}

__global__ void k_f64_to_f32(int64_t n, const double *__restrict__ a, float *__restrict__ b) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}

// ------------------------------------------- factor preconditioner (G^T G) ---
// z = G^T (G r) with G block-lower-triangular on the plan's pattern (the
// learned preconditioner). G is held twice: by rows of its lower part and by
// rows of G^T (the transposed blocks), so both products are row gathers
// (tri_row_acc4).
//
// y = G r (lower rows; rows of pinned vertices give 0) and r.z = r^T G^T G r =
// |y|^2; beta = r.z / r.z_old in the last block.
template <int G>
__global__ void __launch_bounds__(256)
k_pcg_prec_lower(int nV, const int4 *__restrict__ meta, const int *__restrict__ bcol,
                 const __nv_bfloat16 *__restrict__ gl, const float *__restrict__ r, float *__restrict__ y,
                 const unsigned char *__restrict__ pinned, double *__restrict__ part, PcgState *__restrict__ st) {
  pdl_wait();
  pdl_trigger();
  if (st->done) return;
  float acc = 0.f;
  BT_ROW_LOOP_BEGIN(G)
  float s0 = 0.f, s1 = 0.f, s2 = 0.f;
  if (active) {
    const int4 m = __ldg(meta + v);
    const int nl = (m.w & 0xFFFF) + 1;
    tri_row_acc4<G>(sl, bcol + m.x, gl + m.y, 3 * nl, padded_row(nl), [&](int c) { return __ldcg(r + c); }, s0, s1,
                    s2);
  }
  group_reduce<G>(s0, s1, s2);
  if (active && sl == 0) {
    if (pinned && pinned[v]) s0 = s1 = s2 = 0.f;
    y[3 * v] = s0;
    y[3 * v + 1] = s1;
    y[3 * v + 2] = s2;
    acc += s0 * s0 + s1 * s1 + s2 * s2;
  }
  BT_ROW_LOOP_END
  double s = cta_sum_f(acc);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
  if (last_block(&st->count)) {
    const double rz = sum_partials(part, gridDim.x);
    if (threadIdx.x == 0) {
      st->beta = (float)(rz / st->rz);
      st->rz = rz;
      st->count = 0;
    }
  }
}

// z = G^T y (upper rows) and the next direction p = z + beta p_old for the own
// rows (p double-buffered by iteration parity, as k_pcg_dir does).
template <int G>
__global__ void __launch_bounds__(256)
k_pcg_prec_upper(int nV, const int4 *__restrict__ meta, const int *__restrict__ bcol,
                 const __nv_bfloat16 *__restrict__ gu, const float *__restrict__ y, float *__restrict__ pa,
                 float *__restrict__ pb, const unsigned char *__restrict__ pinned, const PcgState *__restrict__ st) {
  pdl_wait();
  pdl_trigger();
  if (st->done) return;
  const int it = st->it;
  const float beta = st->beta;
  const float *p_old = (it & 1) ? pa : pb;
  float *p_new = (it & 1) ? pb : pa;
  BT_ROW_LOOP_BEGIN(G)
  float s0 = 0.f, s1 = 0.f, s2 = 0.f;
  if (active) {
    const int4 m = __ldg(meta + v);
    const int d = m.w & 0xFFFF, nu = (m.w >> 16) - d;
    tri_row_acc4<G>(sl, bcol + m.x + d, gu + m.z, 3 * nu, padded_row(nu), [&](int c) { return __ldcg(y + c); }, s0,
                    s1, s2);
  }
  group_reduce<G>(s0, s1, s2);
  if (active && sl == 0) {
    if (pinned && pinned[v]) s0 = s1 = s2 = 0.f;
    p_new[3 * v] = s0 + beta * __ldcg(p_old + 3 * v);
    p_new[3 * v + 1] = s1 + beta * __ldcg(p_old + 3 * v + 1);
    p_new[3 * v + 2] = s2 + beta * __ldcg(p_old + 3 * v + 2);
  }
  BT_ROW_LOOP_END
}

// x += alpha p; r -= alpha Ap; r.r, iteration count and convergence test
// (the preconditioned residual follows in k_pcg_prec_lower / _upper).
__global__ void __launch_bounds__(256)
k_pcg_update_f(int n, const float *__restrict__ pa, const float *__restrict__ pb, const float *__restrict__ ap,
               float *__restrict__ x, float *__restrict__ r, double *__restrict__ part, PcgState *__restrict__ st) {
  pdl_wait();
  pdl_trigger();
  if (st->done) return;
  const int it = st->it;
  const float *p = (it & 1) ? pb : pa;
  const float alpha = st->alpha;
  float arr = 0.f;
  const int n4 = n / 4;
  const float4 *p4 = reinterpret_cast<const float4 *>(p);
  const float4 *a4 = reinterpret_cast<const float4 *>(ap);
  float4 *x4 = reinterpret_cast<float4 *>(x);
  float4 *r4 = reinterpret_cast<float4 *>(r);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += gridDim.x * blockDim.x) {
    const float4 pv = __ldcg(p4 + i), av = __ldcg(a4 + i);
    float4 xv = x4[i], rv = r4[i];
    xv.x += alpha * pv.x; xv.y += alpha * pv.y; xv.z += alpha * pv.z; xv.w += alpha * pv.w;
    rv.x -= alpha * av.x; rv.y -= alpha * av.y; rv.z -= alpha * av.z; rv.w -= alpha * av.w;
    x4[i] = xv;
    r4[i] = rv;
    arr += rv.x * rv.x + rv.y * rv.y + rv.z * rv.z + rv.w * rv.w;
  }
  for (int i = 4 * n4 + blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    x[i] += alpha * p[i];
    const float rv = r[i] - alpha * ap[i];
    r[i] = rv;
    arr += rv * rv;
  }
  double s = cta_sum_f(arr);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
  if (last_block(&st->count)) {
    const double rr = sum_partials(part, gridDim.x);
    if (threadIdx.x == 0) {
      st->rr = rr;
      st->it = it + 1;
      if (rr <= st->tol2 || it + 1 >= st->max_it || !(rr == rr)) st->done = 1;
      st->count = 0;
    }
  }
}

// start of an inner solve with the factor preconditioner: x = 0, r = rres;
// r.r and the tolerance. A fresh solve (cont = 0) clears p and the iteration
// count (r.z = 1 stands for the previous r.z; beta multiplies p = 0); a
// continued one keeps p, the iteration count and r_k.z_k, so the following
// k_pcg_prec_lower takes beta = r'.z' / r_k.z_k against the replaced residual.
__global__ void k_pcg_init_f(int n, const float *__restrict__ rres, float *__restrict__ x, float *__restrict__ r,
                             float *__restrict__ p0, float *__restrict__ p1, double *__restrict__ part,
                             PcgState *__restrict__ st, double inner_rel2, double abs_tol2, int max_it, int cont) {
  pdl_wait();
  pdl_trigger();
  float arr = 0.f;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float rv = rres[i];
    x[i] = 0.f;
    r[i] = rv;
    if (!cont) {
      p0[i] = 0.f;
      p1[i] = 0.f;
    }
    arr += rv * rv;
  }
  double s = cta_sum_f(arr);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
  if (last_block(&st->count)) {
    const double rr = sum_partials(part, gridDim.x);
    if (threadIdx.x == 0) {
      st->rr = rr;
      st->rr0 = rr;
      if (!cont) st->rz = 1.0;
      else if (!(st->rz > 0.0) || !(st->rz < HUGE_VAL)) st->rz = HUGE_VAL;  // no usable r.z: beta = 0
      st->pap = 0.0;
      st->alpha = 0.f;
      st->beta = 0.f;
      st->tol2 = fmax(inner_rel2 * rr, abs_tol2);
      if (!cont) st->it = 0;
      st->loops = 0;
      st->max_it = st->it + max_it;
      st->done = (rr <= st->tol2 || max_it <= 0 || !(rr == rr)) ? 1 : 0;
      st->count = 0;
    }
  }
}

// ================================================================ host ======
struct PcgOperator {
  // block layout (plan)
  bartels_mesh_plan plan = nullptr;
  const float *values = nullptr;
  const float *vpad = nullptr;    // padded copy of values for the loop's SpMV (nullptr: values' own layout)
  const int *pad_off = nullptr;
  const unsigned char *pinned = nullptr;
  // generic CSR
  int n = 0;
  const int *rp = nullptr, *ci = nullptr;
  const double *values64 = nullptr;  // exact values for the FP64 refinement residual
  // factor preconditioner z = G^T G r (block layout only): lower and upper storage
  const __nv_bfloat16 *gl = nullptr, *gu = nullptr;
  const FactorPattern *fp = nullptr;
  // multigrid V-cycle (block layout only) with its level-0 smoother
  bool mg = false;
  MgSmoother sm;
};

struct PcgWork {
  float *x, *r, *z, *pa, *pb, *ap, *minv, *xh, *xl, *bh, *bl;
  float *rres;  // the refinement residual b - A x (FP32)
  double *part_a, *part_b;
  PcgState *st;
};

static int lanes_spmv(bartels_ctx ctx, bartels_mesh_plan plan) {
  return (plan && plan->spmv_lanes) ? plan->spmv_lanes : ctx->spmv_lanes;
}
static int lanes_tri(bartels_ctx ctx, bartels_mesh_plan plan) {
  return (plan && plan->tri_lanes) ? plan->tri_lanes : ctx->tri_lanes;
}
int plan_lanes_spmv(bartels_ctx ctx, bartels_mesh_plan plan) { return lanes_spmv(ctx, plan); }
int plan_lanes_tri(bartels_ctx ctx, bartels_mesh_plan plan) { return lanes_tri(ctx, plan); }

static int grid_vec(bartels_ctx ctx, int64_t n) {
  int64_t g = (n + 255) / 256;
  int64_t cap = (int64_t)ctx->num_sms * kVecBlocksPerSM;
  return (int)std::max<int64_t>(1, std::min(g, cap));
}
static int grid_spmv(bartels_ctx ctx, int64_t rows) {
  int64_t g = (rows + 7) / 8;  // 8 warps per 256-thread block
  int64_t cap = (int64_t)ctx->num_sms * kSpmvBlocksPerSM;
  return (int)std::max<int64_t>(1, std::min(g, cap));
}
int launch_minv_blk(bartels_ctx ctx, bartels_mesh_plan plan, const float *values, float *minv) {
  BT_LAUNCH(ctx, k_minv_blk, grid_vec(ctx, plan->nV), 256, 0, plan->nV, plan->brp, plan->diag_pos, values,
            plan->pinned, minv);
  return BARTELS_OK;
}


// z = G^T G r, r.z and beta, then p = z + beta p (two launches)
static int pcg_enqueue_prec(bartels_ctx ctx, const PcgOperator &op, const PcgWork &w) {
  const bartels_mesh_plan plan = op.plan;
  // triangular rows are about half as long as the matrix rows (4 or 8 lanes, 4 columns a lane)
  const int G = lanes_tri(ctx, plan);
  const int gt = grid_spmv(ctx, (int64_t)plan->nV * G / 32 + 1);
#define BT_T(G_)                                                                                                 \
  BT_LAUNCH_PDL(ctx, k_pcg_prec_lower<G_>, gt, 256, 0, plan->nV, op.fp->meta, plan->bcol, op.gl, w.r, w.ap, op.pinned, \
            w.part_b, w.st);                                                                                     \
  BT_LAUNCH_PDL(ctx, k_pcg_prec_upper<G_>, gt, 256, 0, plan->nV, op.fp->meta, plan->bcol, op.gu, w.ap, w.pa, w.pb,     \
            op.pinned, w.st)
  if (G == 4) {
    BT_T(4);
  } else {
    BT_T(8);
  }
#undef BT_T
  return BARTELS_OK;
}

// z = B r (V-cycle; its last kernel forms r.z and beta), then p = z + beta p
static int pcg_enqueue_mg(bartels_ctx ctx, const PcgOperator &op, const PcgWork &w, int n, bool pre_done) {
  BT_CHECK(mg_enqueue_apply(ctx, op.plan, op.values, op.sm, w.r, w.z, w.ap, w.part_b, w.st, pre_done));
  BT_LAUNCH_PDL(ctx, k_pcg_dir, grid_vec(ctx, (n + 3) / 4), 256, 0, n, w.z, w.pa, w.pb, w.st);
  return BARTELS_OK;
}

static int pcg_spmv_blk(bartels_ctx ctx, const PcgOperator &op, const PcgWork &w, int lanes, int gs) {
#define BT_K0(G, PAD, VAL, OFF)                                                                                 \
  BT_LAUNCH_PDL(ctx, (k_pcg_spmv_blk<G, PAD>), gs, 256, 0, op.plan->nV, op.plan->brp, op.plan->bcol, VAL, OFF, \
                w.pa, w.pb, w.ap, op.pinned, w.part_a, w.st)
  if (op.vpad) {
    if (lanes == 4) BT_K0(4, true, op.vpad, op.pad_off);
    else if (lanes == 16) BT_K0(16, true, op.vpad, op.pad_off);
    else BT_K0(8, true, op.vpad, op.pad_off);
  } else {
    if (lanes == 4) BT_K0(4, false, op.values, (const int *)nullptr);
    else if (lanes == 16) BT_K0(16, false, op.values, (const int *)nullptr);
    else BT_K0(8, false, op.values, (const int *)nullptr);
  }
#undef BT_K0
  return BARTELS_OK;
}

static int pcg_enqueue_iters(bartels_ctx ctx, const PcgOperator &op, const PcgWork &w, int n, int nb, int iters) {
  const bool blk = op.plan != nullptr;
  const bool fac = blk && op.gl != nullptr;
  const int lanes = blk ? lanes_spmv(ctx, op.plan) : 0;
  const int gs = blk ? grid_spmv(ctx, (int64_t)op.plan->nV * lanes / 32 + 1) : grid_spmv(ctx, n);
  const int gu = grid_vec(ctx, (nb + 3) / 4);
  const int gd = grid_vec(ctx, (n + 3) / 4);
  for (int i = 0; i < iters; ++i) {
    if (op.mg) {
      // p was formed at the end of the previous iteration (or at the start of the solve)
      BT_CHECK(pcg_spmv_blk(ctx, op, w, lanes, gs));
      if (op.sm.gl) {
        BT_LAUNCH_PDL(ctx, k_pcg_update_f, gd, 256, 0, n, w.pa, w.pb, w.ap, w.x, w.r, w.part_b, w.st);
      } else {
        BT_CHECK(mg_enqueue_update(ctx, op.plan, op.sm, w.pa, w.pb, w.ap, w.x, w.r, w.part_b, w.st));
      }
      BT_CHECK(pcg_enqueue_mg(ctx, op, w, n, !op.sm.gl));
      continue;
    }
    // with the factor preconditioner the direction is formed by k_pcg_prec_upper
    if (!fac) BT_LAUNCH_PDL(ctx, k_pcg_dir, gd, 256, 0, n, w.z, w.pa, w.pb, w.st);
    if (blk) {
      BT_CHECK(pcg_spmv_blk(ctx, op, w, lanes, gs));
    } else {
      BT_LAUNCH_PDL(ctx, k_pcg_spmv_csr, gs, 256, 0, n, op.rp, op.ci, op.values, w.pa, w.pb, w.ap, w.part_a, w.st);
    }
    if (fac) {
      BT_LAUNCH_PDL(ctx, k_pcg_update_f, gd, 256, 0, n, w.pa, w.pb, w.ap, w.x, w.r, w.part_b, w.st);
      BT_CHECK(pcg_enqueue_prec(ctx, op, w));
    } else {
      BT_LAUNCH_PDL(ctx, k_pcg_update, gu, 256, 0, nb, n, w.minv, w.pa, w.pb, w.ap, w.x, w.r, w.z, w.part_a, w.part_b,
                w.st);
    }
  }
  return BARTELS_OK;
}

// Loop condition of the device-driven inner solve: a CUDA graph while-node
// whose body is one PCG iteration runs until the solve is done. The body count
// is bounded independently of the iteration count (the iteration cap of the
// state bounds both).
__global__ void k_pcg_cond(cudaGraphConditionalHandle h, PcgState *st) {
  pdl_wait();
  pdl_trigger();
  const unsigned int loops = ++st->loops;
  const bool more = !st->done && st->it < st->max_it && loops <= (unsigned int)st->max_it + 4u;
  cudaGraphSetConditional(h, more ? 1u : 0u);
}

static int launch_cond(bartels_ctx ctx, cudaGraphConditionalHandle h, PcgState *st) {
  BT_LAUNCH_PDL(ctx, k_pcg_cond, 1, 1, 0, h, st);
  return BARTELS_OK;
}

// Executable graph of the inner PCG loop. Preferred: one while-node whose body
// is one iteration (*device_loop = true: a launch runs the inner solve to its
// end with no host round trip and no iteration after convergence). Fallback:
// a fixed run of `chunk` iterations whose kernels turn into no-ops once the
// state is done. *launches: kernel launches per body / chunk.
// BARTELS_PCG_DEVICE_LOOP=0 selects the fixed-length form (kernel profilers
// that replay launches one by one handle plain graphs only).
static bool device_loop_allowed() {
  static const bool allowed = [] {
    const char *e = std::getenv("BARTELS_PCG_DEVICE_LOOP");
    return !(e && e[0] == '0');
  }();
  return allowed;
}

static int build_loop_graph(bartels_ctx ctx, PcgState *st, const std::function<int(int)> &enqueue, int chunk,
                            cudaGraphExec_t *exec, int64_t *launches, bool *device_loop) {
  *exec = nullptr;
  *device_loop = false;
  cudaGraph_t graph = nullptr;
  BT_CUDA(cudaGraphCreate(&graph, 0));
  cudaGraphConditionalHandle h;
  cudaGraphNodeParams cp = {};
  cudaGraphNode_t node;
  cudaError_t e = device_loop_allowed() ? cudaGraphConditionalHandleCreate(&h, graph, 1, cudaGraphCondAssignDefault)
                                        : cudaErrorNotSupported;
  if (e == cudaSuccess) {
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    e = cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &cp);
  }
  if (e == cudaSuccess) {
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    const int64_t before = ctx->launches;
    e = cudaStreamBeginCaptureToGraph(ctx->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      int s = enqueue(1);
      if (s == BARTELS_OK) s = launch_cond(ctx, h, st);
      cudaGraph_t captured = nullptr;
      e = cudaStreamEndCapture(ctx->stream, &captured);
      *launches = ctx->launches - before;
      ctx->launches = before;  // counted per executed body below
      if (s != BARTELS_OK) {
        cudaGraphDestroy(graph);
        return s;
      }
      if (e == cudaSuccess) e = cudaGraphInstantiate(exec, graph, 0);
      cudaGraphDestroy(graph);
      if (e != cudaSuccess) return fail(BARTELS_E_DEVICE, std::string("PCG loop graph: ") + cudaGetErrorString(e));
      *device_loop = true;
      return BARTELS_OK;
    }
  }
  // conditional nodes unavailable: fixed-length graph
  cudaGetLastError();
  cudaGraphDestroy(graph);
  const int64_t before = ctx->launches;
  BT_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  int s = enqueue(chunk);
  e = cudaStreamEndCapture(ctx->stream, &graph);
  *launches = ctx->launches - before;
  ctx->launches = before;  // counted per graph launch below
  if (s != BARTELS_OK) return s;
  if (e != cudaSuccess) return fail(BARTELS_E_DEVICE, std::string("graph capture: ") + cudaGetErrorString(e));
  e = cudaGraphInstantiate(exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return fail(BARTELS_E_DEVICE, std::string("graph instantiate: ") + cudaGetErrorString(e));
  return BARTELS_OK;
}

// Run a full PCG solve of A x = b (FP64 in/out, device pointers) with FP64
// residual refinement. x must be initialised (normally 0).
static int pcg_solve(bartels_ctx ctx, const PcgOperator &op, int n, const double *b, double *x, DevBuf &wbuf,
                     const bartels_pcg_params &prm, bartels_pcg_report *rep) {
  const int nb = (n + 2) / 3;
  const bool blk = op.plan != nullptr;
  const int gs = blk ? grid_spmv(ctx, op.plan->nV) : grid_spmv(ctx, n);
  const int gv = grid_vec(ctx, nb);
  const int nparts = std::max(std::max(gs, gv), 1024);
  // workspace layout
  size_t off = 0;
  auto take = [&](size_t bytes) {
    size_t o = off;
    off += (bytes + 255) & ~size_t(255);
    return o;
  };
  const size_t o_x = take(4ull * n), o_r = take(4ull * n), o_z = take(4ull * n), o_pa = take(4ull * n),
               o_pb = take(4ull * n), o_ap = take(4ull * n), o_minv = take(24ull * nb), o_rres = take(4ull * n),
               o_xh = take(4ull * n), o_xl = take(4ull * n), o_bh = take(4ull * n), o_bl = take(4ull * n),
               o_pa8 = take(8ull * nparts), o_pb8 = take(8ull * nparts), o_st = take(sizeof(PcgState));
  BT_CHECK(wbuf.ensure(off));
  char *base = wbuf.as<char>();
  PcgWork w;
  w.x = (float *)(base + o_x);
  w.r = (float *)(base + o_r);
  w.z = (float *)(base + o_z);
  w.pa = (float *)(base + o_pa);
  w.pb = (float *)(base + o_pb);
  w.ap = (float *)(base + o_ap);
  w.minv = (float *)(base + o_minv);
  w.rres = (float *)(base + o_rres);
  w.bh = (float *)(base + o_bh);
  w.bl = (float *)(base + o_bl);
  w.xh = (float *)(base + o_xh);
  w.xl = (float *)(base + o_xl);
  w.part_a = (double *)(base + o_pa8);
  w.part_b = (double *)(base + o_pb8);
  w.st = (PcgState *)(base + o_st);
  BT_CUDA(cudaMemsetAsync(w.st, 0, sizeof(PcgState), ctx->stream));
  // preconditioner
  if (blk) {
    BT_LAUNCH(ctx, k_minv_blk, grid_vec(ctx, op.plan->nV), 256, 0, op.plan->nV, op.plan->brp, op.plan->diag_pos,
              op.values, op.pinned, w.minv);
  } else {
    BT_LAUNCH(ctx, k_minv_csr, grid_vec(ctx, nb), 256, 0, nb, n, op.rp, op.ci, op.values, w.minv);
  }
  // ||b||
  BT_CHECK(dot(ctx, b, b, n, (double *)&w.st->rr0));
  double bb = 0.0;
  BT_CUDA(cudaMemcpyAsync(&bb, &w.st->rr0, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  BT_CUDA(cudaStreamSynchronize(ctx->stream));
  const double bnorm = std::sqrt(bb);
  rep->iterations = 0;
  rep->refinements = 0;
  rep->converged = 0;
  rep->rel_residual = 0.0;
  if (!(bnorm > 0.0)) {
    BT_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * n, ctx->stream));
    rep->converged = std::isfinite(bnorm) ? 1 : 0;
    return rep->converged ? BARTELS_OK : fail(BARTELS_E_NONFINITE, "non-finite right-hand side");
  }
  const double target = prm.rel_tol * bnorm;
  // CUDA graph of a fixed number of PCG iterations (kernels no-op once done)
  const int chunk = op.mg ? 8 : 16;  // fixed-length fallback only
  cudaGraphExec_t exec = nullptr;
  int64_t graph_launches = 0;
  bool device_loop = false;
  BT_CHECK(build_loop_graph(
      ctx, w.st, [&](int k) { return pcg_enqueue_iters(ctx, op, w, n, nb, k); }, chunk, &exec, &graph_launches,
      &device_loop));
  int status = BARTELS_OK;
  double rel = 0.0;
  PcgState hs{};
  for (int pass = 0; pass <= prm.max_refinements; ++pass) {
    // rres = b - A x (float-float on the block layout, FP64 on a CSR)
    if (blk) {
      if (pass == 0) {
        BT_LAUNCH(ctx, k_axpy64, grid_vec(ctx, n), 256, 0, n, nullptr, x, w.xh, w.xl);
        BT_LAUNCH(ctx, k_split64, grid_vec(ctx, n), 256, 0, n, b, w.bh, w.bl);
      }
      BT_LAUNCH(ctx, k_resid_blk_ff<16>, gs, 256, 0, op.plan->nV, op.plan->brp, op.plan->bcol, op.values, w.xh, w.xl,
                w.bh, w.bl, w.rres, op.pinned, w.part_a);
    } else {
      BT_LAUNCH(ctx, k_resid_csr64, gs, 256, 0, n, op.rp, op.ci, op.values, op.values64, x, b, w.rres, w.part_a);
    }
    BT_CHECK(reduce_sum(ctx, w.part_a, gs, &w.st->rr));
    double rr = 0.0;
    BT_CUDA(cudaMemcpyAsync(&rr, &w.st->rr, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    BT_CUDA(cudaStreamSynchronize(ctx->stream));
    rel = std::sqrt(rr) / bnorm;
    rep->rel_residual = rel;
    if (!std::isfinite(rel)) {
      status = fail(BARTELS_E_NONFINITE, "PCG residual is not finite");
      break;
    }
    if (std::sqrt(rr) <= target) {
      rep->converged = 1;
      break;
    }
    if (pass == prm.max_refinements || rep->iterations >= prm.max_iters) {
      status = fail(BARTELS_E_NOT_CONVERGED, "PCG did not reach the residual target");
      break;
    }
    rep->refinements = pass + 1;
    // inner FP32 PCG on rres: a fresh solve in the first pass, later passes
    // continue the direction against the replaced residual unless restart is set
    const double abs2 = (0.5 * target) * (0.5 * target);
    const int cont = (pass > 0 && !prm.restart) ? 1 : 0;
    const int it0 = cont ? hs.it : 0;
    if (op.mg) {
      BT_LAUNCH_PDL(ctx, k_pcg_init_f, gv, 256, 0, n, w.rres, w.x, w.r, w.pa, w.pb, w.part_a, w.st,
                prm.inner_rel_tol * prm.inner_rel_tol, abs2, prm.max_iters - rep->iterations, cont);
      BT_CHECK(pcg_enqueue_mg(ctx, op, w, n, false));
    } else if (op.gl) {
      BT_LAUNCH_PDL(ctx, k_pcg_init_f, gv, 256, 0, n, w.rres, w.x, w.r, w.pa, w.pb, w.part_a, w.st,
                prm.inner_rel_tol * prm.inner_rel_tol, abs2, prm.max_iters - rep->iterations, cont);
      BT_CHECK(pcg_enqueue_prec(ctx, op, w));
    } else {
      BT_LAUNCH_PDL(ctx, k_pcg_init, gv, 256, 0, nb, n, w.rres, w.minv, w.x, w.r, w.z, w.pa, w.pb, w.part_a, w.part_b,
                w.st, prm.inner_rel_tol * prm.inner_rel_tol, abs2, prm.max_iters - rep->iterations, cont);
    }
    for (;;) {
      BT_CUDA(cudaGraphLaunch(exec, ctx->stream));
      BT_CUDA(cudaMemcpyAsync(&hs, w.st, sizeof(PcgState), cudaMemcpyDeviceToHost, ctx->stream));
      BT_CUDA(cudaStreamSynchronize(ctx->stream));
      if (device_loop) {
        ctx->launches += graph_launches * (int64_t)std::max(1u, hs.loops);
        if (!hs.done) {
          cudaGraphExecDestroy(exec);
          return fail(BARTELS_E_DEVICE, "PCG loop ended before the solve was done");
        }
        break;
      }
      ctx->launches += graph_launches;
      if (hs.done) break;
    }
    rep->iterations += hs.it - it0;
    BT_LAUNCH(ctx, k_axpy64, grid_vec(ctx, n), 256, 0, n, w.x, x, w.xh, w.xl);
  }
  cudaGraphExecDestroy(exec);
  return status;
}

static double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// PCG on a plan's Hessian with the plan's preconditioner. The learned factor is
// built from the current values; when its solve fails (not converged, not
// finite) the system is solved again with block-Jacobi.
// ===================================================== packed meshes ======
// PCG with one set of scalars per segment (an instance of a packed batch):
// alpha_s, beta_s, r.z_s, r.r_s and the convergence test per segment, from
// deterministic per-segment sums (one CTA per segment, fixed order). The
// preconditioners are block diagonal over the segments, so a segment's
// iterates are those it would have alone.
struct SegPtrs {
  int nseg;
  const int *voff, *vseg;
  double *rz, *rr, *tol2, *abs2, *red;
  float *alpha, *beta;
  int *done, *iters;
};

enum { kSegNorm = 0, kSegInit = 1, kSegPap = 2, kSegRzRr = 3 };

// Per-segment sums a.b (and c.d) and the scalars of MODE:
//   kSegNorm: red_s = a.b;
//   kSegInit: r.z_s = a.b, r.r_s = c.d, tol2_s, done_s (also set by the host
//             for segments that need no iterations), beta_s = 0;
//   kSegPap:  alpha_s = r.z_s / (p.Ap)_s with p taken by iteration parity;
//   kSegRzRr: beta_s = r.z'_s / r.z_s, r.z_s, r.r_s, done_s, iteration count.
// kSegInit and kSegRzRr end with the last CTA setting the global state (all
// segments done, or the iteration cap) that the shared kernels and the loop
// condition read.
template <int MODE>
__global__ void __launch_bounds__(256)
k_seg_scalars(SegPtrs sp, const float *__restrict__ a, const float *__restrict__ b, const float *__restrict__ c,
              const float *__restrict__ d, const float *__restrict__ pa, const float *__restrict__ pb, double inner2,
              int max_it, PcgState *__restrict__ st) {
  pdl_wait();
  pdl_trigger();
  if ((MODE == kSegPap || MODE == kSegRzRr) && st->done) return;
  if (MODE == kSegPap) a = (st->it & 1) ? pb : pa;
  const int s = blockIdx.x;
  const int i0 = 3 * sp.voff[s], i1 = 3 * sp.voff[s + 1];
  float acc1 = 0.f, acc2 = 0.f;
  for (int i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
    acc1 += __ldcg(a + i) * __ldcg(b + i);
    if (c) acc2 += __ldcg(c + i) * __ldcg(d + i);
  }
  const double s1 = cta_sum_f(acc1);
  const double s2 = c ? cta_sum_f(acc2) : 0.0;
  if (threadIdx.x == 0) {
    if (MODE == kSegNorm) {
      sp.red[s] = s1;
    } else if (MODE == kSegInit) {
      const bool skip = sp.done[s] != 0;
      sp.rz[s] = s1;
      sp.rr[s] = s2;
      sp.tol2[s] = fmax(inner2 * s2, sp.abs2[s]);
      sp.alpha[s] = 0.f;
      sp.beta[s] = 0.f;
      sp.done[s] = (skip || s2 <= sp.tol2[s] || !(s2 == s2)) ? 1 : 0;
    } else if (MODE == kSegPap) {
      sp.alpha[s] = sp.done[s] ? 0.f : (float)(sp.rz[s] / s1);
    } else {
      if (!sp.done[s]) {
        sp.beta[s] = (float)(s1 / sp.rz[s]);
        sp.rz[s] = s1;
        sp.rr[s] = s2;
        sp.iters[s] += 1;
        if (s2 <= sp.tol2[s] || !(s2 == s2)) sp.done[s] = 1;
      } else {
        sp.beta[s] = 0.f;
      }
    }
  }
  if (MODE == kSegInit || MODE == kSegRzRr) {
    if (last_block(&st->count)) {
      int all = 1;
      for (int q = threadIdx.x; q < sp.nseg; q += blockDim.x)
        if (!__ldcg(sp.done + q)) all = 0;
      all = __syncthreads_and(all);
      if (threadIdx.x == 0) {
        if (MODE == kSegInit) {
          st->it = 0;
          st->max_it = max_it;
          st->loops = 0;
          st->done = (all || max_it <= 0) ? 1 : 0;
        } else {
          st->it += 1;
          st->done = (all || st->it >= st->max_it) ? 1 : 0;
        }
        st->count = 0;
      }
    }
  }
}

// start of a pass: x = 0, r = rres (0 in segments that take no iterations),
// z = M^-1 r with block-Jacobi (multigrid computes z afterwards), p = 0; the
// global state reopened for the kernels that follow
__global__ void __launch_bounds__(256)
k_seg_init(int nV, const int *__restrict__ vseg, const int *__restrict__ done, const float *__restrict__ rres,
           const float *__restrict__ minv, float *__restrict__ x, float *__restrict__ r, float *__restrict__ z,
           float *__restrict__ p0, float *__restrict__ p1, PcgState *__restrict__ st) {
  pdl_wait();
  pdl_trigger();
  if (blockIdx.x == 0 && threadIdx.x == 0) st->done = 0;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nV; v += gridDim.x * blockDim.x) {
    const bool skip = done[vseg[v]] != 0;
    float rv[3], zv[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      rv[k] = skip ? 0.f : rres[3 * v + k];
      x[3 * v + k] = 0.f;
      r[3 * v + k] = rv[k];
      p0[3 * v + k] = 0.f;
      p1[3 * v + k] = 0.f;
    }
    if (minv) {
      apply_minv(minv, v, rv, zv);
#pragma unroll
      for (int k = 0; k < 3; ++k) z[3 * v + k] = zv[k];
    }
  }
}

// x += alpha_s p; r -= alpha_s Ap; z = M^-1 r with block-Jacobi (minv), per vertex with its segment's step
__global__ void __launch_bounds__(256)
k_seg_update(int nV, const int *__restrict__ vseg, const float *__restrict__ alpha, const float *__restrict__ pa,
             const float *__restrict__ pb, const float *__restrict__ ap, float *__restrict__ x, float *__restrict__ r,
             float *__restrict__ z, const float *__restrict__ minv, const PcgState *__restrict__ st) {
  pdl_wait();
  pdl_trigger();
  if (st->done) return;
  const float *p = (st->it & 1) ? pb : pa;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nV; v += gridDim.x * blockDim.x) {
    const float al = alpha[vseg[v]];
    float rv[3], zv[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const int i = 3 * v + k;
      x[i] += al * __ldcg(p + i);
      rv[k] = r[i] - al * __ldcg(ap + i);
      r[i] = rv[k];
    }
    if (minv) {
      apply_minv(minv, v, rv, zv);
#pragma unroll
      for (int k = 0; k < 3; ++k) z[3 * v + k] = zv[k];
    }
  }
}

// p = z + beta_s p_old (double-buffered by iteration parity, as k_pcg_dir)
__global__ void __launch_bounds__(256)
k_seg_dir(int nV, const int *__restrict__ vseg, const float *__restrict__ beta, const float *__restrict__ z,
          float *__restrict__ pa, float *__restrict__ pb, const PcgState *__restrict__ st) {
  pdl_wait();
  pdl_trigger();
  if (st->done) return;
  const int it = st->it;
  const float *p_old = (it & 1) ? pa : pb;
  float *p_new = (it & 1) ? pb : pa;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nV; v += gridDim.x * blockDim.x) {
    const float bt = beta[vseg[v]];
#pragma unroll
    for (int k = 0; k < 3; ++k) p_new[3 * v + k] = __ldcg(z + 3 * v + k) + bt * __ldcg(p_old + 3 * v + k);
  }
}

// per-segment FP64 sums a.b (or of a alone when b is NULL) over the entries
// [mult voff[s], mult voff[s + 1]) (vertex offsets: mult = 3 for DOF vectors,
// 1 for per-vertex values) or [eoff[s], eoff[s + 1]) (tet offsets)
__global__ void __launch_bounds__(256)
k_seg_dot64(const int *__restrict__ voff, int mult, const int64_t *__restrict__ eoff, const double *__restrict__ a,
            const double *__restrict__ b, double *__restrict__ out) {
  const int s = blockIdx.x;
  const int64_t i0 = eoff ? eoff[s] : (int64_t)mult * voff[s], i1 = eoff ? eoff[s + 1] : (int64_t)mult * voff[s + 1];
  double acc = 0.0;
  for (int64_t i = i0 + threadIdx.x; i < i1; i += blockDim.x) acc += b ? a[i] * b[i] : a[i];
  const double t = cta_sum(acc);
  if (threadIdx.x == 0) out[s] = t;
}

// x += alpha_s d per vertex (FP64)
__global__ void k_seg_axpy(int nV, const int *__restrict__ vseg, const double *__restrict__ alpha,
                           const double *__restrict__ d, double *__restrict__ x) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nV; v += gridDim.x * blockDim.x) {
    const double al = alpha[vseg[v]];
    for (int k = 0; k < 3; ++k) x[3 * v + k] += al * d[3 * v + k];
  }
}

static SegPtrs seg_ptrs(const SegInfo *sg) {
  SegPtrs sp;
  sp.nseg = sg->nseg;
  sp.voff = sg->voff;
  sp.vseg = sg->vseg;
  sp.rz = sg->rz;
  sp.rr = sg->rr;
  sp.tol2 = sg->tol2;
  sp.abs2 = sg->abs2;
  sp.red = sg->red;
  sp.alpha = sg->alpha;
  sp.beta = sg->beta;
  sp.done = sg->done;
  sp.iters = sg->iters;
  return sp;
}

// One PCG iteration of the segmented solve (or `iters` of them).
static int seg_enqueue_iters(bartels_ctx ctx, const PcgOperator &op, const PcgWork &w, const SegPtrs &sp, int iters) {
  const bartels_mesh_plan plan = op.plan;
  const int nV = plan->nV;
  const int lanes = lanes_spmv(ctx, plan);
  const int gs = grid_spmv(ctx, (int64_t)nV * lanes / 32 + 1);
  const int gv = grid_vec(ctx, nV);
  for (int i = 0; i < iters; ++i) {
    BT_CHECK(pcg_spmv_blk(ctx, op, w, lanes, gs));
    BT_LAUNCH_PDL(ctx, k_seg_scalars<kSegPap>, sp.nseg, 256, 0, sp, (const float *)nullptr, w.ap,
                  (const float *)nullptr, (const float *)nullptr, w.pa, w.pb, 0.0, 0, w.st);
    BT_LAUNCH_PDL(ctx, k_seg_update, gv, 256, 0, nV, sp.vseg, sp.alpha, w.pa, w.pb, w.ap, w.x, w.r, w.z,
                  op.mg ? (const float *)nullptr : w.minv, w.st);
    if (op.mg) BT_CHECK(mg_enqueue_apply(ctx, plan, op.values, op.sm, w.r, w.z, w.ap, w.part_b, w.st, false));
    BT_LAUNCH_PDL(ctx, k_seg_scalars<kSegRzRr>, sp.nseg, 256, 0, sp, w.r, w.z, w.r, w.r, (const float *)nullptr,
                  (const float *)nullptr, 0.0, 0, w.st);
    BT_LAUNCH_PDL(ctx, k_seg_dir, gv, 256, 0, nV, sp.vseg, sp.beta, w.z, w.pa, w.pb, w.st);
  }
  return BARTELS_OK;
}

// A full solve of A x = b over the plan's segments (FP64 in / out, device),
// FP64 residual refinement per segment: each pass computes b - A x (float-
// float), and the segments whose residual is still above rel_tol of their own
// |b_s| (and that are active) take a restarted inner FP32 PCG to inner_rel_tol.
static int seg_pcg_solve(bartels_ctx ctx, const PcgOperator &op, const double *b, double *x, DevBuf &wbuf,
                         const bartels_pcg_params &prm, bartels_pcg_report *rep) {
  const bartels_mesh_plan plan = op.plan;
  SegInfo *sg = plan->seg;
  const int nseg = sg->nseg, nV = plan->nV, n = 3 * nV;
  const int gs = grid_spmv(ctx, nV);
  const int gv = grid_vec(ctx, nV);
  const int nparts = std::max(std::max(gs, gv), 1024);
  size_t off = 0;
  auto take = [&](size_t bytes) {
    size_t o = off;
    off += (bytes + 255) & ~size_t(255);
    return o;
  };
  const size_t o_x = take(4ull * n), o_r = take(4ull * n), o_z = take(4ull * n), o_pa = take(4ull * n),
               o_pb = take(4ull * n), o_ap = take(4ull * n), o_minv = take(24ull * nV), o_rres = take(4ull * n),
               o_xh = take(4ull * n), o_xl = take(4ull * n), o_bh = take(4ull * n), o_bl = take(4ull * n),
               o_pa8 = take(8ull * nparts), o_pb8 = take(8ull * nparts), o_st = take(sizeof(PcgState));
  BT_CHECK(wbuf.ensure(off));
  char *base = wbuf.as<char>();
  PcgWork w;
  w.x = (float *)(base + o_x);
  w.r = (float *)(base + o_r);
  w.z = (float *)(base + o_z);
  w.pa = (float *)(base + o_pa);
  w.pb = (float *)(base + o_pb);
  w.ap = (float *)(base + o_ap);
  w.minv = (float *)(base + o_minv);
  w.rres = (float *)(base + o_rres);
  w.bh = (float *)(base + o_bh);
  w.bl = (float *)(base + o_bl);
  w.xh = (float *)(base + o_xh);
  w.xl = (float *)(base + o_xl);
  w.part_a = (double *)(base + o_pa8);
  w.part_b = (double *)(base + o_pb8);
  w.st = (PcgState *)(base + o_st);
  BT_CUDA(cudaMemsetAsync(w.st, 0, sizeof(PcgState), ctx->stream));
  BT_CUDA(cudaMemsetAsync(sg->iters, 0, sizeof(int) * nseg, ctx->stream));
  if (!op.mg) BT_LAUNCH(ctx, k_minv_blk, grid_vec(ctx, nV), 256, 0, nV, plan->brp, plan->diag_pos, op.values,
                        op.pinned, w.minv);
  const SegPtrs sp = seg_ptrs(sg);
  // |b_s|
  BT_LAUNCH(ctx, k_seg_dot64, nseg, 256, 0, sg->voff, 3, (const int64_t *)nullptr, b, b, sg->red2);
  std::vector<double> bn(nseg), rr(nseg), abs2(nseg);
  std::vector<int> skip(nseg);
  BT_CUDA(cudaMemcpyAsync(bn.data(), sg->red2, sizeof(double) * nseg, cudaMemcpyDeviceToHost, ctx->stream));
  BT_CUDA(cudaStreamSynchronize(ctx->stream));
  for (int q = 0; q < nseg; ++q) {
    bn[q] = std::sqrt(bn[q]);
    abs2[q] = (0.5 * prm.rel_tol * bn[q]) * (0.5 * prm.rel_tol * bn[q]);
  }
  BT_CUDA(cudaMemcpyAsync(sg->abs2, abs2.data(), sizeof(double) * nseg, cudaMemcpyHostToDevice, ctx->stream));
  cudaGraphExec_t exec = nullptr;
  int64_t graph_launches = 0;
  bool device_loop = false;
  BT_CHECK(build_loop_graph(
      ctx, w.st, [&](int k) { return seg_enqueue_iters(ctx, op, w, sp, k); }, 8, &exec, &graph_launches,
      &device_loop));
  rep->iterations = 0;
  rep->refinements = 0;
  rep->converged = 0;
  rep->rel_residual = 0.0;
  int status = BARTELS_OK;
  PcgState hs{};
  const int lanes_r = 16;
  for (int pass = 0; pass <= prm.max_refinements; ++pass) {
    if (pass == 0) {
      BT_LAUNCH(ctx, k_axpy64, grid_vec(ctx, n), 256, 0, n, nullptr, x, w.xh, w.xl);
      BT_LAUNCH(ctx, k_split64, grid_vec(ctx, n), 256, 0, n, b, w.bh, w.bl);
    }
    BT_LAUNCH(ctx, k_resid_blk_ff<lanes_r>, gs, 256, 0, nV, plan->brp, plan->bcol, op.values, w.xh, w.xl, w.bh,
              w.bl, w.rres, op.pinned, w.part_a);
    BT_LAUNCH(ctx, k_seg_scalars<kSegNorm>, nseg, 256, 0, sp, w.rres, w.rres, (const float *)nullptr,
              (const float *)nullptr, (const float *)nullptr, (const float *)nullptr, 0.0, 0, w.st);
    BT_CUDA(cudaMemcpyAsync(rr.data(), sg->red, sizeof(double) * nseg, cudaMemcpyDeviceToHost, ctx->stream));
    BT_CUDA(cudaStreamSynchronize(ctx->stream));
    double rel = 0.0;
    int work = 0;
    bool finite = true;
    for (int q = 0; q < nseg; ++q) {
      const double r = std::sqrt(rr[q]);
      if (!std::isfinite(r)) finite = false;
      const double rq = bn[q] > 0.0 ? r / bn[q] : 0.0;
      const bool need = sg->active[q] && bn[q] > 0.0 && r > prm.rel_tol * bn[q];
      skip[q] = need ? 0 : 1;
      work += need;
      if (sg->active[q]) rel = std::max(rel, rq);
    }
    rep->rel_residual = rel;
    if (!finite) {
      status = fail(BARTELS_E_NONFINITE, "PCG residual is not finite");
      break;
    }
    if (work == 0) {
      rep->converged = 1;
      break;
    }
    if (pass == prm.max_refinements || rep->iterations >= prm.max_iters) {
      status = fail(BARTELS_E_NOT_CONVERGED, "PCG did not reach the residual target");
      break;
    }
    rep->refinements = pass + 1;
    BT_CUDA(cudaMemcpyAsync(sg->done, skip.data(), sizeof(int) * nseg, cudaMemcpyHostToDevice, ctx->stream));
    BT_LAUNCH_PDL(ctx, k_seg_init, gv, 256, 0, nV, sg->vseg, sg->done, w.rres, op.mg ? (const float *)nullptr : w.minv,
                  w.x, w.r, w.z, w.pa, w.pb, w.st);
    if (op.mg) BT_CHECK(mg_enqueue_apply(ctx, plan, op.values, op.sm, w.r, w.z, w.ap, w.part_b, w.st, false));
    BT_LAUNCH_PDL(ctx, k_seg_scalars<kSegInit>, nseg, 256, 0, sp, w.r, w.z, w.r, w.r, (const float *)nullptr,
                  (const float *)nullptr, prm.inner_rel_tol * prm.inner_rel_tol, prm.max_iters - rep->iterations,
                  w.st);
    BT_LAUNCH_PDL(ctx, k_seg_dir, gv, 256, 0, nV, sg->vseg, sg->beta, w.z, w.pa, w.pb, w.st);
    for (;;) {
      BT_CUDA(cudaGraphLaunch(exec, ctx->stream));
      BT_CUDA(cudaMemcpyAsync(&hs, w.st, sizeof(PcgState), cudaMemcpyDeviceToHost, ctx->stream));
      BT_CUDA(cudaStreamSynchronize(ctx->stream));
      if (device_loop) {
        ctx->launches += graph_launches * (int64_t)std::max(1u, hs.loops);
        break;
      }
      ctx->launches += graph_launches;
      if (hs.done) break;
    }
    rep->iterations += hs.it;
    BT_LAUNCH(ctx, k_axpy64, grid_vec(ctx, n), 256, 0, n, w.x, x, w.xh, w.xl);
  }
  cudaGraphExecDestroy(exec);
  sg->last_iters.resize(nseg);
  BT_CUDA(cudaMemcpyAsync(sg->last_iters.data(), sg->iters, sizeof(int) * nseg, cudaMemcpyDeviceToHost, ctx->stream));
  BT_CUDA(cudaStreamSynchronize(ctx->stream));
  return status;
}

// Multigrid hierarchy values for a Hessian: the level-0 smoother (block-Jacobi
// inverse blocks, or the network's factor), Galerkin products, bounds.
static int mg_values(bartels_ctx ctx, bartels_mesh_plan plan, const float *values, bool learned, MgSmoother &sm) {
  sm = MgSmoother();
  if (learned) {
    BT_CHECK(lpcg_factor(plan->lpcg_net, plan, values, &sm.gl, &sm.gu));
    sm.fp = plan->factor;
  } else {
    BT_CHECK(plan->w_minv.ensure(24 * (size_t)plan->nV));
    BT_CHECK(launch_minv_blk(ctx, plan, values, plan->w_minv.as<float>()));
    sm.minv = plan->w_minv.as<float>();
  }
  return mg_setup_numeric(ctx, plan, values, sm);
}

int plan_precond_apply(bartels_ctx ctx, bartels_mesh_plan plan, const float *values, const float *r, float *z,
                       int *levels) {
  const bool learned = plan->precond == BARTELS_PRECOND_LEARNED_MULTIGRID && plan->lpcg_net;
  if (plan->precond != BARTELS_PRECOND_MULTIGRID && !learned)
    return fail(BARTELS_E_INVALID_ARG, "the plan's preconditioner is not a multigrid one");
  BT_CHECK(mg_prepare(ctx, plan));
  MgSmoother sm;
  BT_CHECK(mg_values(ctx, plan, values, learned, sm));
  BT_CHECK(mg_apply_once(ctx, plan, values, sm, r, z));
  if (levels) *levels = (int)plan->mg->lv.size();
  return BARTELS_OK;
}

SegInfo::~SegInfo() {
  for (void *q : allocs) cudaFree(q);
}

// Segments of a packed plan: offsets checked (monotone, covering the mesh,
// every tet inside its segment), per-vertex and per-tet segment maps and the
// per-segment scalar buffers.
int plan_set_segments(bartels_mesh_plan plan, int nseg, const int *voff, const int64_t *toff) {
  delete plan->seg;
  plan->seg = nullptr;
  if (nseg == 0) return BARTELS_OK;
  if (nseg < 0 || !voff || !toff) return fail(BARTELS_E_INVALID_ARG, "bad segment arguments");
  if (voff[0] != 0 || voff[nseg] != plan->nV || toff[0] != 0 || toff[nseg] != plan->nT)
    return fail(BARTELS_E_INVALID_ARG, "segment offsets must start at 0 and end at the vertex / tet counts");
  for (int q = 0; q < nseg; ++q)
    if (voff[q + 1] < voff[q] || toff[q + 1] < toff[q])
      return fail(BARTELS_E_INVALID_ARG, "segment offsets must not decrease");
  std::vector<int4> E(plan->nT);
  BT_CUDA(cudaMemcpy(E.data(), plan->E, sizeof(int4) * E.size(), cudaMemcpyDeviceToHost));
  std::vector<int> vseg(plan->nV), tseg(plan->nT);
  for (int q = 0; q < nseg; ++q) {
    for (int v = voff[q]; v < voff[q + 1]; ++v) vseg[v] = q;
    for (int64_t t = toff[q]; t < toff[q + 1]; ++t) {
      tseg[t] = q;
      const int id[4] = {E[t].x, E[t].y, E[t].z, E[t].w};
      for (int a = 0; a < 4; ++a)
        if (id[a] < voff[q] || id[a] >= voff[q + 1])
          return fail(BARTELS_E_INVALID_ARG, "tet " + std::to_string(t) + " has a vertex outside its segment");
    }
  }
  auto *sg = new SegInfo();
  plan->seg = sg;
  sg->nseg = nseg;
  sg->h_voff.assign(voff, voff + nseg + 1);
  sg->h_toff.assign(toff, toff + nseg + 1);
  sg->active.assign(nseg, 1);
  auto alloc = [&](void **dst, size_t bytes) -> int {
    BT_CUDA(cudaMalloc(dst, std::max<size_t>(bytes, 16)));
    sg->allocs.push_back(*dst);
    return BARTELS_OK;
  };
  BT_CHECK(alloc((void **)&sg->voff, sizeof(int) * (nseg + 1)));
  BT_CHECK(alloc((void **)&sg->toff, sizeof(int64_t) * (nseg + 1)));
  BT_CHECK(alloc((void **)&sg->vseg, sizeof(int) * plan->nV));
  BT_CHECK(alloc((void **)&sg->tseg, sizeof(int) * plan->nT));
  for (double **d : {&sg->rz, &sg->rr, &sg->tol2, &sg->abs2, &sg->red, &sg->red2, &sg->alpha64})
    BT_CHECK(alloc((void **)d, sizeof(double) * nseg));
  BT_CHECK(alloc((void **)&sg->alpha, sizeof(float) * nseg));
  BT_CHECK(alloc((void **)&sg->beta, sizeof(float) * nseg));
  BT_CHECK(alloc((void **)&sg->done, sizeof(int) * nseg));
  BT_CHECK(alloc((void **)&sg->iters, sizeof(int) * nseg));
  BT_CHECK(alloc((void **)&sg->et, sizeof(double) * plan->nT));
  BT_CHECK(alloc((void **)&sg->ev, sizeof(double) * plan->nV));
  BT_CUDA(cudaMemcpy(sg->voff, voff, sizeof(int) * (nseg + 1), cudaMemcpyHostToDevice));
  BT_CUDA(cudaMemcpy(sg->toff, toff, sizeof(int64_t) * (nseg + 1), cudaMemcpyHostToDevice));
  BT_CUDA(cudaMemcpy(sg->vseg, vseg.data(), sizeof(int) * plan->nV, cudaMemcpyHostToDevice));
  BT_CUDA(cudaMemcpy(sg->tseg, tseg.data(), sizeof(int) * plan->nT, cudaMemcpyHostToDevice));
  return BARTELS_OK;
}

// The PCG loop's SpMV reads a padded copy of the values (three scalar rows
// per vertex, each padded with zeros to a multiple of 4 entries, so that a
// lane reads 4 values with one 16-byte load); the copy is made once per
// linear solve. BARTELS_PCG_PADDED=0 keeps the values' own layout.
static bool padded_spmv_enabled() {
  static const bool on = [] {
    const char *e = std::getenv("BARTELS_PCG_PADDED");
    return !(e && e[0] == '0');
  }();
  return on;
}

static int plan_pad_offsets(bartels_mesh_plan plan) {
  if (plan->pad_off) return BARTELS_OK;
  std::vector<int> off(plan->nV + 1, 0);
  for (int v = 0; v < plan->nV; ++v) {
    const int64_t next = off[v] + 3ll * padded_row(plan->h_brp[v + 1] - plan->h_brp[v]);
    if (next > INT_MAX) return fail(BARTELS_E_UNSUPPORTED, "padded values larger than 2^31 entries");
    off[v + 1] = (int)next;
  }
  BT_CUDA(cudaMalloc(&plan->pad_off, sizeof(int) * off.size()));
  BT_CUDA(cudaMemcpy(plan->pad_off, off.data(), sizeof(int) * off.size(), cudaMemcpyHostToDevice));
  plan->pad_total = off[plan->nV];
  return BARTELS_OK;
}

// *out = the padded copy of values (nullptr when the padded SpMV is off)
static int plan_padded_values(bartels_ctx ctx, bartels_mesh_plan plan, const float *values, const float **out) {
  *out = nullptr;
  if (!padded_spmv_enabled() || !values) return BARTELS_OK;
  BT_CHECK(plan_pad_offsets(plan));
  const size_t bytes = sizeof(float) * ((size_t)plan->pad_total + 4);
  if (plan->w_vpad.bytes < bytes) {
    BT_CHECK(plan->w_vpad.ensure(bytes));
    BT_CUDA(cudaMemsetAsync(plan->w_vpad.p, 0, plan->w_vpad.bytes, ctx->stream));
  }
  BT_LAUNCH(ctx, k_pad_values, grid_spmv(ctx, plan->nV), 256, 0, plan->nV, plan->brp, (const int *)plan->pad_off,
            values, plan->w_vpad.as<float>());
  *out = plan->w_vpad.as<float>();
  return BARTELS_OK;
}

// The plan's solve: per-segment scalars for packed meshes (block-Jacobi or a
// multigrid V-cycle; the single-level factor preconditioner runs as block-
// Jacobi there), one system otherwise.
static int solve_any(bartels_ctx ctx, PcgOperator op, int n, const double *b, double *x, DevBuf &wbuf,
                     const bartels_pcg_params &prm, bartels_pcg_report *rep) {
  if (op.plan && op.plan->seg && op.plan->seg->nseg > 0) {
    op.gl = op.gu = nullptr;
    op.fp = nullptr;
    return seg_pcg_solve(ctx, op, b, x, wbuf, prm, rep);
  }
  return pcg_solve(ctx, op, n, b, x, wbuf, prm, rep);
}

static int plan_pcg_impl(bartels_ctx ctx, bartels_mesh_plan plan, const float *values, const double *b, double *x,
                         const bartels_pcg_params &prm, bartels_pcg_report *rep, int *fallback, double *t_factor) {
  const int n = 3 * plan->nV;
  PcgOperator op;
  op.plan = plan;
  op.values = values;
  op.pinned = plan->pinned;
  BT_CHECK(plan_padded_values(ctx, plan, values, &op.vpad));
  op.pad_off = plan->pad_off;
  if (fallback) *fallback = 0;
  const bool mg_learned = plan->precond == BARTELS_PRECOND_LEARNED_MULTIGRID && plan->lpcg_net;
  if (plan->precond == BARTELS_PRECOND_MULTIGRID || mg_learned) {
    const double t0 = now_s();
    int s = mg_prepare(ctx, plan);
    if (s != BARTELS_OK && s != BARTELS_E_UNSUPPORTED) return s;
    if (s == BARTELS_OK) {
      MgSmoother sm;
      BT_CHECK(mg_values(ctx, plan, values, mg_learned, sm));
      BT_CUDA(cudaStreamSynchronize(ctx->stream));
      if (t_factor) *t_factor += now_s() - t0;
      op.mg = true;
      op.sm = sm;
      // a multigrid solve needs tens to a few hundred iterations on these
      // systems; one that has not converged after kMgMaxIters has stagnated and
      // moves on to the next preconditioner instead of running to the caller's cap
      constexpr int kMgMaxIters = 1500;
      bartels_pcg_params prm_mg = prm;
      prm_mg.max_iters = std::min(prm.max_iters, kMgMaxIters);
      s = solve_any(ctx, op, n, b, x, plan->w_pcg, prm_mg, rep);
      if (s == BARTELS_OK && rep->converged) return BARTELS_OK;
      if (s != BARTELS_OK && s != BARTELS_E_NOT_CONVERGED && s != BARTELS_E_NONFINITE) return s;
      if (fallback) *fallback = 1;
      int used = rep->iterations;
      if (mg_learned) {
        // the learned smoother failed this system: the same V-cycle with
        // block-Jacobi smoothing first (a block-Jacobi solve costs ~25x the
        // iterations on these systems)
        MgSmoother bj;
        BT_CHECK(mg_values(ctx, plan, values, false, bj));
        op.sm = bj;
        BT_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * n, ctx->stream));
        s = solve_any(ctx, op, n, b, x, plan->w_pcg, prm_mg, rep);
        rep->iterations += used;
        if (s == BARTELS_OK && rep->converged) return BARTELS_OK;
        if (s != BARTELS_OK && s != BARTELS_E_NOT_CONVERGED && s != BARTELS_E_NONFINITE) return s;
        used = rep->iterations;
      }
      // not converged or not finite: solve again with block-Jacobi
      op.mg = false;
      op.sm = MgSmoother();
      BT_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * n, ctx->stream));
      s = solve_any(ctx, op, n, b, x, plan->w_pcg, prm, rep);
      rep->iterations += used;
      return s;
    }
    // a system too small for a coarse level: block-Jacobi
    set_error("");
  }
  if (plan->precond == BARTELS_PRECOND_LEARNED && plan->lpcg_net) {
    const double t0 = now_s();
    const __nv_bfloat16 *gl = nullptr, *gu = nullptr;
    BT_CHECK(lpcg_factor(plan->lpcg_net, plan, values, &gl, &gu));
    BT_CUDA(cudaStreamSynchronize(ctx->stream));
    if (t_factor) *t_factor += now_s() - t0;
    op.gl = gl;
    op.gu = gu;
    op.fp = plan->factor;
    int s = solve_any(ctx, op, n, b, x, plan->w_pcg, prm, rep);
    if (s == BARTELS_OK && rep->converged) return BARTELS_OK;
    if (s != BARTELS_OK && s != BARTELS_E_NOT_CONVERGED && s != BARTELS_E_NONFINITE) return s;
    if (fallback) *fallback = 1;
    const int used = rep->iterations;
    op.gl = op.gu = nullptr;
    op.fp = nullptr;
    BT_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * n, ctx->stream));
    s = solve_any(ctx, op, n, b, x, plan->w_pcg, prm, rep);
    rep->iterations += used;
    return s;
  }
  return solve_any(ctx, op, n, b, x, plan->w_pcg, prm, rep);
}

int plan_pcg(bartels_ctx ctx, bartels_mesh_plan plan, const float *values, const double *b, double *x,
             const bartels_pcg_params &prm, bartels_pcg_report *rep) {
  BT_CUDA(cudaMemsetAsync(x, 0, sizeof(double) * 3 * (size_t)plan->nV, ctx->stream));
  return plan_pcg_impl(ctx, plan, values, b, x, prm, rep, nullptr, nullptr);
}

// ============================================================ Newton =======
struct NewtonWork {
  double *g, *d, *xt, *scal;
  float4 *u;
  float *values;
};

static int newton_work(bartels_mesh_plan plan, NewtonWork &w) {
  const size_t n = 3 * (size_t)plan->nV;
  BT_CHECK(plan->w_vec.ensure(sizeof(double) * (3 * n + 16)));
  BT_CHECK(plan->w_u.ensure(2 * sizeof(float4) * (size_t)plan->nV));
  BT_CHECK(plan->w_values.ensure(sizeof(float) * 9 * (size_t)plan->nnzb));
  double *b = plan->w_vec.as<double>();
  w.g = b;
  w.d = b + n;
  w.xt = b + 2 * n;
  w.scal = b + 3 * n;
  w.u = plan->w_u.as<float4>();
  w.values = plan->w_values.as<float>();
  return BARTELS_OK;
}

static ObjectiveDev objective_of(bartels_mesh_plan plan, const bartels_newton_params &p) {
  ObjectiveDev o;
  o.mass_coeff = p.mass_coeff;
  o.scale = p.scale;
  o.force_scale = p.force_scale;
  o.q_base = plan->q_base;
  o.x_hat = plan->x_hat;
  o.f_ext = plan->f_ext;
  o.pinned = plan->pinned;
  return o;
}

static int read_scalar(bartels_ctx ctx, const double *d, double *h) {
  BT_CUDA(cudaMemcpyAsync(ctx->host_scalars, d, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  BT_CUDA(cudaStreamSynchronize(ctx->stream));
  *h = ctx->host_scalars[0];
  return BARTELS_OK;
}

// NVTX range per Newton stage (gradient, Hessian, PCG, line search) for
// timeline profilers; the range open at a return is closed by the destructor.
// Without a profiler attached each call is a check of one function pointer.
struct NvtxStage {
  bool open = false;
  void to(const char *name) {
    if (open) nvtxRangePop();
    nvtxRangePushA(name);
    open = true;
  }
  ~NvtxStage() {
    if (open) nvtxRangePop();
  }
};

// The reference's line search (src/linesearch_backtracking_bisection.cpp:17-30)
// for every segment of a packed plan at once, each with its own step: segment
// s accepts alpha_s when f_s(x + alpha_s d) - f_s(x) <= c g_s.d_s, else halves
// it (up to max_iterations_ls times); inactive segments take no step.
static int seg_linesearch(bartels_ctx ctx, bartels_mesh_plan plan, const bartels_newton_params &p,
                          const ObjectiveDev &obj, double *x, const NewtonWork &w, bartels_newton_report *rep) {
  SegInfo *sg = plan->seg;
  const int nseg = sg->nseg;
  BT_LAUNCH(ctx, k_seg_dot64, nseg, 256, 0, sg->voff, 3, (const int64_t *)nullptr, w.g, w.d, sg->red2);
  std::vector<double> gd(nseg), alpha(nseg), trial(nseg), det(nseg), dev(nseg);
  std::vector<int> searching(nseg), back(nseg, 0);
  BT_CUDA(cudaMemcpyAsync(gd.data(), sg->red2, sizeof(double) * nseg, cudaMemcpyDeviceToHost, ctx->stream));
  BT_CUDA(cudaStreamSynchronize(ctx->stream));
  for (int q = 0; q < nseg; ++q) {
    searching[q] = sg->active[q] ? 1 : 0;
    alpha[q] = sg->active[q] ? p.ls_alpha : 0.0;
  }
  double df_total = 0.0;
  for (int it = 0;; ++it) {
    int any = 0;
    for (int q = 0; q < nseg; ++q) {
      trial[q] = searching[q] ? alpha[q] : 0.0;
      any += searching[q];
    }
    if (!any) break;
    BT_CUDA(cudaMemcpyAsync(sg->alpha64, trial.data(), sizeof(double) * nseg, cudaMemcpyHostToDevice, ctx->stream));
    BT_CHECK(energy_diff_seg(ctx, plan, p.model, obj, x, w.d, sg->alpha64, sg->tseg, sg->vseg, sg->et, sg->ev));
    BT_LAUNCH(ctx, k_seg_dot64, nseg, 256, 0, (const int *)nullptr, 0, sg->toff, sg->et, (const double *)nullptr,
              sg->red);
    BT_LAUNCH(ctx, k_seg_dot64, nseg, 256, 0, sg->voff, 1, (const int64_t *)nullptr, sg->ev, (const double *)nullptr,
              sg->red2);
    BT_CUDA(cudaMemcpyAsync(det.data(), sg->red, sizeof(double) * nseg, cudaMemcpyDeviceToHost, ctx->stream));
    BT_CUDA(cudaMemcpyAsync(dev.data(), sg->red2, sizeof(double) * nseg, cudaMemcpyDeviceToHost, ctx->stream));
    BT_CUDA(cudaStreamSynchronize(ctx->stream));
    for (int q = 0; q < nseg; ++q) {
      if (!searching[q]) continue;
      const double df = det[q] + dev[q];
      const bool reject = !std::isfinite(df) || df > p.ls_c * gd[q];
      if (reject && it < p.max_iterations_ls) {
        alpha[q] *= p.ls_p;
        back[q]++;
      } else {
        searching[q] = 0;
        if (reject) rep->ls_failures++;
        else df_total += df;
      }
    }
  }
  BT_CUDA(cudaMemcpyAsync(sg->alpha64, alpha.data(), sizeof(double) * nseg, cudaMemcpyHostToDevice, ctx->stream));
  BT_LAUNCH(ctx, k_seg_axpy, grid_vec(ctx, plan->nV), 256, 0, plan->nV, sg->vseg, sg->alpha64, w.d, x);
  int most = 0;
  double amin = HUGE_VAL;
  for (int q = 0; q < nseg; ++q) {
    most = std::max(most, back[q]);
    if (sg->active[q]) amin = std::min(amin, alpha[q]);
  }
  rep->ls_iterations += most;
  rep->last_alpha = amin < HUGE_VAL ? amin : 0.0;
  rep->energy_change = df_total;
  return BARTELS_OK;
}

int newton_iterate(bartels_ctx ctx, bartels_mesh_plan plan, const bartels_newton_params &p, double *x,
                   double g0_norm, int *done, bartels_newton_report *rep) {
  NvtxStage stage;
  stage.to("bartels newton: gradient");
  NewtonWork w;
  BT_CHECK(newton_work(plan, w));
  const int n = 3 * plan->nV;
  const ObjectiveDev obj = objective_of(plan, p);
  double t0 = now_s();
  // gradient and convergence test (include/optimization_gradient_based.h:80-84)
  BT_CHECK(gradient(ctx, plan, p.model, obj, x, w.g));
  BT_CHECK(dot(ctx, w.g, w.g, n, w.scal));
  double gg;
  BT_CHECK(read_scalar(ctx, w.scal, &gg));
  double t1 = now_s();
  rep->t_gradient += t1 - t0;
  const double gnorm = std::sqrt(gg);
  rep->grad_norm = gnorm;
  if (!std::isfinite(gnorm)) return fail(BARTELS_E_NONFINITE, "gradient is not finite (inverted element?)");
  const bool conv = p.relative ? (gnorm <= p.gradient_tol * g0_norm) : (gg < p.gradient_tol * p.gradient_tol);
  if (conv) {
    *done = 1;
    return BARTELS_OK;
  }
  *done = 0;
  stage.to("bartels newton: hessian");
  // Hessian H = mass_coeff M + scale^2 K (fused assembly, FP32)
  BT_CHECK(launch_prep_u(ctx, plan, x, plan->q_base, p.scale, plan->dphi_matches_rest, w.u));
  BT_CHECK(launch_hess(ctx, plan, p.model, p.psd_mode, w.u, plan->dphi_matches_rest ? 1 : 0,
                       (float)(p.scale * p.scale), (float)p.mass_coeff, (float)p.psd_tol, p.dq2_flags, w.values));
  BT_CUDA(cudaStreamSynchronize(ctx->stream));
  double t2 = now_s();
  rep->t_hessian += t2 - t1;
  stage.to("bartels newton: pcg");
  // search direction d = -H^-1 g (src/search_direction_newton_sparse.cpp:12-24)
  BT_LAUNCH(ctx, k_scale_copy, grid_vec(ctx, n), 256, 0, n, -1.0, w.g, w.xt);
  BT_CUDA(cudaMemsetAsync(w.d, 0, sizeof(double) * n, ctx->stream));
  bartels_pcg_report pr;
  int fb = 0;
  int s = plan_pcg_impl(ctx, plan, w.values, w.xt, w.d, p.pcg, &pr, &fb, &rep->t_precond);
  rep->precond_fallbacks += fb;
  rep->pcg_iterations += pr.iterations;
  rep->last_pcg_iterations = pr.iterations;
  rep->last_pcg_refinements = pr.refinements;
  rep->last_pcg_rel_residual = pr.rel_residual;
  if (!pr.converged) rep->pcg_failures++;
  double t3 = now_s();
  rep->t_pcg += t3 - t2;
  if (s != BARTELS_OK && s != BARTELS_E_NOT_CONVERGED) return s;
  stage.to("bartels newton: line search");
  // line search (src/linesearch_backtracking_bisection.cpp:17-30): while
  // f(x + alpha d) > f(x) + c g.d and it < max: alpha *= p. The difference
  // f(x + alpha d) - f(x) is evaluated element by element (energy_diff) so that
  // it stays accurate when it is many orders below |f| near the minimum.
  if (plan->seg && plan->seg->nseg > 0) {
    BT_CHECK(seg_linesearch(ctx, plan, p, obj, x, w, rep));
    BT_CUDA(cudaStreamSynchronize(ctx->stream));
    rep->t_linesearch += now_s() - t3;
    rep->iterations += 1;
    return BARTELS_OK;
  }
  double gd;
  BT_CHECK(dot(ctx, w.g, w.d, n, w.scal));
  BT_CHECK(read_scalar(ctx, w.scal, &gd));
  double alpha = p.ls_alpha;
  int it = 0;
  double df = 0.0;
  for (;;) {
    BT_CHECK(energy_diff(ctx, plan, p.model, obj, x, w.d, alpha, w.scal));
    BT_CHECK(read_scalar(ctx, w.scal, &df));
    // the reference's test (a NaN energy, e.g. from an inverted Neo-Hookean
    // element, also backtracks instead of being accepted)
    const bool reject = !std::isfinite(df) || df > p.ls_c * gd;
    if (!(reject && it < p.max_iterations_ls)) break;
    alpha *= p.ls_p;
    it++;
  }
  BT_LAUNCH(ctx, k_axpy_to, grid_vec(ctx, n), 256, 0, n, x, alpha, w.d, w.xt);
  rep->energy_change = df;
  if (it == p.max_iterations_ls) rep->ls_failures++;
  rep->last_alpha = alpha;
  BT_CUDA(cudaMemcpyAsync(x, w.xt, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->stream));
  rep->ls_iterations += it;
  BT_CUDA(cudaStreamSynchronize(ctx->stream));
  rep->t_linesearch += now_s() - t3;
  rep->iterations += 1;
  return BARTELS_OK;
}

int newton_gradient(bartels_ctx ctx, bartels_mesh_plan plan, const bartels_newton_params &p, const double *x,
                    double *g) {
  return gradient(ctx, plan, p.model, objective_of(plan, p), x, g);
}

int newton_energy(bartels_ctx ctx, bartels_mesh_plan plan, const bartels_newton_params &p, const double *x,
                  double *energy_host) {
  NewtonWork w;
  BT_CHECK(newton_work(plan, w));
  BT_CHECK(energy(ctx, plan, p.model, objective_of(plan, p), x, w.scal));
  return read_scalar(ctx, w.scal, energy_host);
}

int newton_solve(bartels_ctx ctx, bartels_mesh_plan plan, const bartels_newton_params &p, double *x,
                 bartels_newton_report *rep) {
  const double t0 = now_s();
  NewtonWork w;
  BT_CHECK(newton_work(plan, w));
  const int n = 3 * plan->nV;
  const ObjectiveDev obj = objective_of(plan, p);
  // reference gradient norm for the relative test
  BT_CHECK(gradient(ctx, plan, p.model, obj, x, w.g));
  BT_CHECK(dot(ctx, w.g, w.g, n, w.scal));
  double gg;
  BT_CHECK(read_scalar(ctx, w.scal, &gg));
  rep->grad_norm0 = std::sqrt(gg);
  rep->status = BARTELS_MAX_ITERATIONS_REACHED;
  int count = 0;
  do {
    int done = 0;
    BT_CHECK(newton_iterate(ctx, plan, p, x, rep->grad_norm0, &done, rep));
    if (done) {
      rep->status = BARTELS_CONVERGED;
      break;
    }
    count++;
  } while (count <= p.max_iterations);
  double f;
  BT_CHECK(energy(ctx, plan, p.model, obj, x, w.scal));
  BT_CHECK(read_scalar(ctx, w.scal, &f));
  rep->energy = f;
  rep->seconds = now_s() - t0;
  return BARTELS_OK;
}

__global__ void k_advance_ie(int n, double dt, const double *__restrict__ v, double *__restrict__ q_base,
                             double *__restrict__ x_hat) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    q_base[i] += dt * v[i];
    x_hat[i] = v[i];
  }
}

int advance_implicit_euler(bartels_ctx ctx, bartels_mesh_plan plan, double dt, const double *v) {
  const int n = 3 * plan->nV;
  if (!plan->q_base) {
    BT_CUDA(cudaMalloc(&plan->q_base, sizeof(double) * n));
    BT_CUDA(cudaMemsetAsync(plan->q_base, 0, sizeof(double) * n, ctx->stream));
  }
  if (!plan->x_hat) BT_CUDA(cudaMalloc(&plan->x_hat, sizeof(double) * n));
  BT_LAUNCH(ctx, k_advance_ie, grid_vec(ctx, n), 256, 0, n, dt, v, plan->q_base, plan->x_hat);
  return BARTELS_OK;
}

// y = A x with the PCG loop's own SpMV kernel (k_pcg_spmv_blk, which also
// forms the partial sums of x.Ax), on a scratch state of the plan, so that
// timing this entry point times the SpMV the solves run. The state is zeroed
// once when its buffer is made; the kernel's last block resets its counter.
int plan_spmv(bartels_ctx ctx, bartels_mesh_plan plan, const float *values, const float *x, float *y) {
  const int lanes = lanes_spmv(ctx, plan);
  const int g = grid_spmv(ctx, (int64_t)plan->nV * lanes / 32 + 1);
  const size_t o_st = (sizeof(double) * g + 255) & ~size_t(255);
  const size_t need = o_st + sizeof(PcgState);
  if (plan->w_spmv.bytes < need) {
    BT_CHECK(plan->w_spmv.ensure(need));
    BT_CUDA(cudaMemsetAsync(plan->w_spmv.p, 0, plan->w_spmv.bytes, ctx->stream));
  }
  double *part = plan->w_spmv.as<double>();
  PcgState *st = reinterpret_cast<PcgState *>(plan->w_spmv.as<char>() + o_st);
#define BT_SPMV(G)                                                                                               \
  BT_LAUNCH_PDL(ctx, (k_pcg_spmv_blk<G, false>), g, 256, 0, plan->nV, plan->brp, plan->bcol, values, (const int *)nullptr, \
                x, x, y, plan->pinned, part, st)
  if (lanes == 4) BT_SPMV(4);
  else if (lanes == 16) BT_SPMV(16);
  else BT_SPMV(8);
#undef BT_SPMV
  return BARTELS_OK;
}

// The PCG loop's SpMV kernel on these values (over the padded copy when the
// loop uses one, made once here), y = A x: 3 warm-up launches, then reps
// launches timed with CUDA events on the context's stream; *us = microseconds
// per launch.
int plan_pcg_spmv_time(bartels_ctx ctx, bartels_mesh_plan plan, const float *values, const float *x, float *y,
                       int reps, double *us) {
  const int lanes = lanes_spmv(ctx, plan);
  const int g = grid_spmv(ctx, (int64_t)plan->nV * lanes / 32 + 1);
  const size_t o_st = (sizeof(double) * g + 255) & ~size_t(255);
  const size_t need = o_st + sizeof(PcgState);
  if (plan->w_spmv.bytes < need) {
    BT_CHECK(plan->w_spmv.ensure(need));
    BT_CUDA(cudaMemsetAsync(plan->w_spmv.p, 0, plan->w_spmv.bytes, ctx->stream));
  }
  double *part = plan->w_spmv.as<double>();
  PcgState *st = reinterpret_cast<PcgState *>(plan->w_spmv.as<char>() + o_st);
  const float *vpad = nullptr;
  BT_CHECK(plan_padded_values(ctx, plan, values, &vpad));
  const int *poff = plan->pad_off;
  const int nV = plan->nV;
  auto launch = [&]() {
#define BT_TL(GG)                                                                                                  \
  do {                                                                                                             \
    if (vpad)                                                                                                      \
      k_pcg_spmv_blk<GG, true><<<g, 256, 0, ctx->stream>>>(nV, plan->brp, plan->bcol, vpad, poff, x, x, y,         \
                                                           plan->pinned, part, st);                                \
    else                                                                                                           \
      k_pcg_spmv_blk<GG, false><<<g, 256, 0, ctx->stream>>>(nV, plan->brp, plan->bcol, values, nullptr, x, x, y,   \
                                                            plan->pinned, part, st);                               \
  } while (0)
    if (lanes == 4) BT_TL(4);
    else if (lanes == 16) BT_TL(16);
    else BT_TL(8);
#undef BT_TL
  };
  cudaEvent_t e0, e1;
  BT_CUDA(cudaEventCreate(&e0));
  BT_CUDA(cudaEventCreate(&e1));
  for (int k = 0; k < 3; ++k) launch();
  cudaEventRecord(e0, ctx->stream);
  for (int k = 0; k < reps; ++k) launch();
  cudaEventRecord(e1, ctx->stream);
  cudaError_t e = cudaEventSynchronize(e1);
  float ms = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  if (e == cudaSuccess) e = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (e != cudaSuccess) return fail(BARTELS_E_DEVICE, std::string("SpMV timing: ") + cudaGetErrorString(e));
  ctx->launches += 3 + reps;
  *us = 1e3 * ms / reps;
  return BARTELS_OK;
}

// Hessian autotuner: time the fused PSD-projected assembly at positions q
// (3 warm-up + 5 timed calls, CUDA events on the context's stream, best of
// three rounds over the candidates) for every
// pair of assembly CTA shape (128 vertices / 64 KB or 64 vertices / 32 KB of
// shared memory) and PSD pre-pass block size (64, 128, 256 threads); keep the
// fastest in the plan and in the context's cache for the size bucket
// floor(log2 nV), which later plans of that bucket take without timing. The
// assembled values do not depend on the choice (each entry is still summed by
// its row's thread in tet order).
int plan_autotune_hessian(bartels_ctx ctx, bartels_mesh_plan plan, int model, const double *q, int force,
                          int *chunk_out, int *block_out) {
  int bucket = 0;
  for (int v = plan->nV; v > 1; v >>= 1) bucket++;
  auto hit = ctx->tune_cache_hess.find(bucket);
  if (!force && hit != ctx->tune_cache_hess.end()) {
    if (hit->second.first == 64) BT_CHECK(plan_chunks64(plan));
    plan->hess_chunk = hit->second.first;
    plan->psd_block = hit->second.second;
  } else {
    // the half-size chunks exist unless a vertex row needs more than their shared memory
    const bool have64 = plan_chunks64(plan) == BARTELS_OK;
    BT_CHECK(plan->w_u.ensure(2 * sizeof(float4) * (size_t)plan->nV));
    BT_CHECK(plan->w_values.ensure(sizeof(float) * 9 * (size_t)plan->nnzb));
    float *vals = plan->w_values.as<float>();
    float4 *u = plan->w_u.as<float4>();
    BT_CHECK(launch_prep_u(ctx, plan, q, nullptr, 1.0, plan->dphi_matches_rest, u));
    cudaEvent_t e0, e1;
    BT_CUDA(cudaEventCreate(&e0));
    BT_CUDA(cudaEventCreate(&e1));
    float tbest[2][3];
    for (auto &row : tbest)
      for (float &t : row) t = 1e30f;
    int bc = 128, bb = 128;
    int status = BARTELS_OK;
    const int chunks[2] = {128, 64}, blocks[3] = {64, 128, 256};
    // three rounds over the candidates, each one's best time kept (clock ramp-up)
    for (int round = 0; round < 3; ++round)
    for (int ci = 0; ci < 2; ++ci)
      for (int bi = 0; bi < 3; ++bi) {
        const int c = chunks[ci], bl = blocks[bi];
        if (c == 64 && !have64) continue;
        plan->hess_chunk = c;
        plan->psd_block = bl;
        for (int k = 0; k < 8 && status == BARTELS_OK; ++k) {
          if (k == 3) cudaEventRecord(e0, ctx->stream);
          status = launch_hess(ctx, plan, model, BARTELS_PSD_SIMPLE_FIX, u, plan->dphi_matches_rest ? 1 : 0, 1.f,
                               0.f, 1e-6f, 0, vals);
        }
        cudaEventRecord(e1, ctx->stream);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (status == BARTELS_OK) tbest[ci][bi] = std::min(tbest[ci][bi], ms);
      }
    {
      float b = 1e30f;
      for (int ci = 0; ci < 2; ++ci)
        for (int bi = 0; bi < 3; ++bi)
          if (tbest[ci][bi] < b) b = tbest[ci][bi], bc = chunks[ci], bb = blocks[bi];
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (status != BARTELS_OK) return status;
    plan->hess_chunk = bc;
    plan->psd_block = bb;
    ctx->tune_cache_hess[bucket] = {bc, bb};
  }
  if (chunk_out) *chunk_out = plan->hess_chunk;
  if (block_out) *block_out = plan->psd_block;
  return BARTELS_OK;
}

int plan_set_hessian_tuning(bartels_mesh_plan plan, int chunk, int block) {
  if ((chunk != 64 && chunk != 128) || (block != 64 && block != 128 && block != 256))
    return fail(BARTELS_E_INVALID_ARG, "assembly CTA shape must be 64 or 128 vertices, PSD block 64, 128 or 256");
  if (chunk == 64) BT_CHECK(plan_chunks64(plan));
  plan->hess_chunk = chunk;
  plan->psd_block = block;
  return BARTELS_OK;
}

// Autotuner: time the PCG loop's block-row SpMV with 4, 8 and 16 lanes per
// vertex row and the factor passes with 4 and 8 lanes on this plan (CUDA
// events on the context's stream, 3 warm-up + 10 timed launches each, best of
// three rounds over the candidates), keep the fastest in
// the plan and in the context's cache for the plan's size bucket
// floor(log2 nV), which later plans of that bucket reuse without timing.
int plan_autotune(bartels_ctx ctx, bartels_mesh_plan plan, const float *values, int force, int *spmv_out,
                  int *tri_out) {
  int bucket = 0;
  for (int v = plan->nV; v > 1; v >>= 1) bucket++;
  auto hit = ctx->tune_cache.find(bucket);
  if (!force && hit != ctx->tune_cache.end()) {
    plan->spmv_lanes = hit->second.first;
    plan->tri_lanes = hit->second.second;
  } else {
    FactorPattern *fp;
    BT_CHECK(plan_factor_pattern(plan, &fp));
    const size_t n = 3 * (size_t)plan->nV;
    float *x = nullptr, *y = nullptr;
    __nv_bfloat16 *gl = nullptr;
    PcgState *st = nullptr;
    double *part = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int status = BARTELS_OK;
    auto cleanup = [&]() {
      if (x) cudaFree(x);
      if (y) cudaFree(y);
      if (gl) cudaFree(gl);
      if (st) cudaFree(st);
      if (part) cudaFree(part);
      if (e0) cudaEventDestroy(e0);
      if (e1) cudaEventDestroy(e1);
    };
    auto timed = [&](auto &&launch) -> float {
      for (int k = 0; k < 3; ++k) launch();
      cudaEventRecord(e0, ctx->stream);
      for (int k = 0; k < 10; ++k) launch();
      cudaEventRecord(e1, ctx->stream);
      cudaEventSynchronize(e1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      return ms;
    };
    if (cudaMalloc(&x, 4 * n) != cudaSuccess || cudaMalloc(&y, 4 * n) != cudaSuccess ||
        cudaMalloc(&gl, 2 * (size_t)fp->lsize + 16) != cudaSuccess || cudaMalloc(&st, sizeof(PcgState)) != cudaSuccess ||
        cudaMalloc(&part, 8 * 4096) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
        cudaEventCreate(&e1) != cudaSuccess) {
      cleanup();
      return fail(BARTELS_E_DEVICE, "autotuner scratch allocation failed");
    }
    cudaMemsetAsync(x, 0, 4 * n, ctx->stream);
    cudaMemsetAsync(gl, 0, 2 * (size_t)fp->lsize + 16, ctx->stream);
    cudaMemsetAsync(st, 0, sizeof(PcgState), ctx->stream);
    const int nV = plan->nV;
    const float *vpad = nullptr;
    const int ps = plan_padded_values(ctx, plan, values, &vpad);
    if (ps != BARTELS_OK) {
      cleanup();
      return ps;  // with plan_padded_values' message
    }
    const int *poff = plan->pad_off;
    // three rounds over the candidates, each candidate's best time kept (the
    // clocks may still be ramping up when a plan is set up)
    constexpr int kRounds = 3;
    float t_s[3] = {1e30f, 1e30f, 1e30f}, t_t[2] = {1e30f, 1e30f};
    int best_s = ctx->spmv_lanes, best_t = ctx->tri_lanes;
    const int cand_s[3] = {4, 8, 16};
    for (int round = 0; round < kRounds; ++round)
    for (int ci = 0; ci < 3; ++ci) {
      const int G = cand_s[ci];
      const int g = grid_spmv(ctx, (int64_t)nV * G / 32 + 1);
      // the PCG loop's own SpMV (A p and the partials of p.Ap) on a scratch state
      const float ms = timed([&] {
#define BT_TS(GG)                                                                                             \
  do {                                                                                                        \
    if (vpad)                                                                                                 \
      k_pcg_spmv_blk<GG, true><<<g, 256, 0, ctx->stream>>>(nV, plan->brp, plan->bcol, vpad, poff, x, x, y,    \
                                                           plan->pinned, part, st);                           \
    else                                                                                                      \
      k_pcg_spmv_blk<GG, false><<<g, 256, 0, ctx->stream>>>(nV, plan->brp, plan->bcol, values, nullptr, x, x, \
                                                            y, plan->pinned, part, st);                       \
  } while (0)
        if (G == 4) BT_TS(4);
        else if (G == 8) BT_TS(8);
        else BT_TS(16);
#undef BT_TS
      });
      t_s[ci] = std::min(t_s[ci], ms);
    }
    const int cand_t[2] = {4, 8};
    for (int round = 0; round < kRounds; ++round)
    for (int ci = 0; ci < 2; ++ci) {
      const int G = cand_t[ci];
      const int g = grid_spmv(ctx, (int64_t)nV * G / 32 + 1);
      const float ms = timed([&] {
        if (G == 4)
          k_pcg_prec_lower<4><<<g, 256, 0, ctx->stream>>>(nV, fp->meta, plan->bcol, gl, x, y, plan->pinned, part, st);
        else
          k_pcg_prec_lower<8><<<g, 256, 0, ctx->stream>>>(nV, fp->meta, plan->bcol, gl, x, y, plan->pinned, part, st);
      });
      t_t[ci] = std::min(t_t[ci], ms);
    }
    {
      float b = 1e30f;
      for (int ci = 0; ci < 3; ++ci)
        if (t_s[ci] < b) b = t_s[ci], best_s = cand_s[ci];
      b = 1e30f;
      for (int ci = 0; ci < 2; ++ci)
        if (t_t[ci] < b) b = t_t[ci], best_t = cand_t[ci];
    }
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e == cudaSuccess) e = cudaGetLastError();
    cleanup();
    if (e != cudaSuccess) status = fail(BARTELS_E_DEVICE, std::string("autotuner: ") + cudaGetErrorString(e));
    if (status != BARTELS_OK) return status;
    ctx->launches += 39 * kRounds;
    plan->spmv_lanes = best_s;
    plan->tri_lanes = best_t;
    ctx->tune_cache[bucket] = {best_s, best_t};
  }
  if (spmv_out) *spmv_out = plan->spmv_lanes;
  if (tri_out) *tri_out = plan->tri_lanes;
  return BARTELS_OK;
}

// out[s] = sum over the DOFs of vertices off[s] .. off[s+1]-1 of v^2 (one block per segment)
__global__ void __launch_bounds__(256)
k_segment_sumsq(int nseg, const int *__restrict__ off, const double *__restrict__ v, double *__restrict__ out) {
  for (int sgm = blockIdx.x; sgm < nseg; sgm += gridDim.x) {
    double acc = 0.0;
    for (int64_t i = 3ll * off[sgm] + threadIdx.x; i < 3ll * off[sgm + 1]; i += blockDim.x) acc += v[i] * v[i];
    const double s = cta_sum(acc);
    if (threadIdx.x == 0) out[sgm] = s;
  }
}

int segment_sumsq(bartels_ctx ctx, int nseg, const int *off, const double *v, double *out) {
  if (nseg <= 0) return BARTELS_OK;
  BT_LAUNCH(ctx, k_segment_sumsq, std::min(nseg, 65535), 256, 0, nseg, off, v, out);
  return BARTELS_OK;
}

// generic CSR solve for the drop-in search direction
int csr_search_direction(bartels_ctx ctx, int n, const int *rp, const int *ci, const double *vals, const double *g,
                         double *d, const bartels_pcg_params &prm, bartels_pcg_report *rep) {
  const int64_t nnz = (n > 0) ? rp[n] : 0;
  size_t bytes_rp = sizeof(int) * (n + 1), bytes_ci = sizeof(int) * nnz, bytes_v64 = sizeof(double) * nnz;
  BT_CHECK(ctx->stage_a.ensure(bytes_rp + bytes_ci + 512));
  BT_CHECK(ctx->stage_b.ensure(bytes_v64 + sizeof(float) * nnz + 512));
  BT_CHECK(ctx->stage_c.ensure(sizeof(double) * 2 * (size_t)n + 512));
  int *drp = ctx->stage_a.as<int>();
  int *dci = drp + ((n + 1 + 63) & ~63);
  double *dv64 = ctx->stage_b.as<double>();
  float *dv32 = reinterpret_cast<float *>(dv64 + ((nnz + 63) & ~63ll));
  double *db = ctx->stage_c.as<double>();
  double *dx = db + ((n + 63) & ~63);
  BT_CUDA(cudaMemcpyAsync(drp, rp, bytes_rp, cudaMemcpyHostToDevice, ctx->stream));
  BT_CUDA(cudaMemcpyAsync(dci, ci, bytes_ci, cudaMemcpyHostToDevice, ctx->stream));
  BT_CUDA(cudaMemcpyAsync(dv64, vals, bytes_v64, cudaMemcpyHostToDevice, ctx->stream));
  BT_CUDA(cudaMemcpyAsync(dx, g, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
  BT_LAUNCH(ctx, k_f64_to_f32, grid_vec(ctx, nnz), 256, 0, nnz, dv64, dv32);
  BT_LAUNCH(ctx, k_scale_copy, grid_vec(ctx, n), 256, 0, n, -1.0, dx, db);
  BT_CUDA(cudaMemsetAsync(dx, 0, sizeof(double) * n, ctx->stream));
  PcgOperator op;
  op.n = n;
  op.rp = drp;
  op.ci = dci;
  op.values = dv32;
  op.values64 = dv64;
  int s = pcg_solve(ctx, op, n, db, dx, ctx->stage_d, prm, rep);
  BT_CUDA(cudaMemcpyAsync(d, dx, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
  BT_CUDA(cudaStreamSynchronize(ctx->stream));
  return s;
}

}  // namespace bartels
