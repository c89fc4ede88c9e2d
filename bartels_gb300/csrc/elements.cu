// Element kernels of the tet-mesh path: shape-function gradients and volumes,
// per-tet records, FP64 energy and gradient, and the fused FP32 Hessian
// assembly (element math + PSD projection + deterministic per-row sums in tet
// order, written straight into the CSR value array).
#include <algorithm>
#include <mutex>
#include <string>

#include "devmath.cuh"
#include "internal.cuh"

namespace bartels {

// ---------------------------------------------------------------- helpers ---
__device__ __forceinline__ void load_rec32(const TetRec32 *__restrict__ rec, int t, TetRec32 &r) {
  const float4 *p = reinterpret_cast<const float4 *>(rec + t);
  float4 a = __ldg(p + 0), b = __ldg(p + 1), c = __ldg(p + 2), d = __ldg(p + 3);
  r.idx = make_int4(__float_as_int(a.x), __float_as_int(a.y), __float_as_int(a.z), __float_as_int(a.w));
  r.dphi[0] = b.x; r.dphi[1] = b.y; r.dphi[2] = b.z; r.dphi[3] = b.w;
  r.dphi[4] = c.x; r.dphi[5] = c.y; r.dphi[6] = c.z; r.dphi[7] = c.w;
  r.dphi[8] = d.x; r.pv[0] = d.y; r.pv[1] = d.z; r.mass = d.w;
}

template <class T>
__device__ __forceinline__ void phi4(const T *dphi9, T (*phi)[3]) {
  for (int d = 0; d < 3; ++d) {
    phi[1][d] = dphi9[d];
    phi[2][d] = dphi9[3 + d];
    phi[3][d] = dphi9[6 + d];
    phi[0][d] = -(phi[1][d] + phi[2][d] + phi[3][d]);
  }
}

// block reduction of one double per thread into out (fixed order)
__device__ __forceinline__ double block_sum(double v) {
  __shared__ double red[32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) red[w] = v;
  __syncthreads();
  double s = 0.0;
  if (w == 0) {
    const int nw = (blockDim.x + 31) >> 5;
    s = lane < nw ? red[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  }
  __syncthreads();
  return s;  // valid in thread 0
}

// ------------------------------------------------------------- kinematics ---
// linear_tet_dphi_dX (src/linear_tet_dphi_dX.cpp:10-16) and signed volume, one
// thread per tet in FP64. Writes the reference's nT x 12 column-major layout
// (optional), the internal rows 1..3 (dphi9) and the volume.
__global__ void k_dphi_vol(int nT, const double *__restrict__ X, const int4 *__restrict__ E,
                           double *__restrict__ dphidX_cm, double *__restrict__ dphi9, double *__restrict__ vol) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nT; t += gridDim.x * blockDim.x) {
    int4 e = E[t];
    const int id[4] = {e.x, e.y, e.z, e.w};
    double Dm[9];
    for (int c = 0; c < 3; ++c)
      for (int d = 0; d < 3; ++d) Dm[d + 3 * c] = X[3 * id[c + 1] + d] - X[3 * id[0] + d];
    double G[9];
    cof3(G, Dm);
    double det = Dm[0] * G[0] + Dm[1] * G[1] + Dm[2] * G[2];
    double inv = 1.0 / det;
    // inverse = G^T / det; row (a-1) of the inverse is phi_a
    double phi[4][3];
    for (int a = 1; a < 4; ++a)
      for (int d = 0; d < 3; ++d) phi[a][d] = G[d + 3 * (a - 1)] * inv;
    for (int d = 0; d < 3; ++d) phi[0][d] = -(phi[1][d] + phi[2][d] + phi[3][d]);
    if (dphidX_cm)
      for (int a = 0; a < 4; ++a)
        for (int d = 0; d < 3; ++d) dphidX_cm[t + (size_t)nT * (a + 4 * d)] = phi[a][d];
    if (dphi9)
      for (int a = 1; a < 4; ++a)
        for (int d = 0; d < 3; ++d) dphi9[9ll * t + 3 * (a - 1) + d] = phi[a][d];
    if (vol) vol[t] = det / 6.0;
  }
}

// Import a caller's nT x 12 column-major dphidX. err[0] collects the largest
// |phi_0 + phi_1 + phi_2 + phi_3| relative to |phi| (must be ~0: the plan
// stores rows 1..3 only), err[1] the largest |sum_a (X_a - X_0) phi_a^T - I|
// (0 when dphidX belongs to the plan's rest shape).
__global__ void k_import_dphi(int nT, const double *__restrict__ src, const double *__restrict__ X,
                              const int4 *__restrict__ E, double *__restrict__ dphi9, double *__restrict__ err) {
  double e0 = 0.0, e1 = 0.0;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nT; t += gridDim.x * blockDim.x) {
    double phi[4][3], mag = 0.0;
    for (int a = 0; a < 4; ++a)
      for (int d = 0; d < 3; ++d) {
        phi[a][d] = src[t + (size_t)nT * (a + 4 * d)];
        mag = fmax(mag, fabs(phi[a][d]));
      }
    for (int d = 0; d < 3; ++d) {
      double s = phi[0][d] + phi[1][d] + phi[2][d] + phi[3][d];
      e0 = fmax(e0, fabs(s) / (mag > 0 ? mag : 1.0));
    }
    for (int a = 1; a < 4; ++a)
      for (int d = 0; d < 3; ++d) dphi9[9ll * t + 3 * (a - 1) + d] = phi[a][d];
    int4 e = E[t];
    const int id[4] = {e.x, e.y, e.z, e.w};
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        double s = (i == j) ? -1.0 : 0.0;
        for (int a = 1; a < 4; ++a) s += (X[3 * id[a] + i] - X[3 * id[0] + i]) * phi[a][j];
        e1 = fmax(e1, fabs(s));
      }
  }
  // max-reduce with atomics on the bit pattern of non-negative doubles
  for (int o = 16; o > 0; o >>= 1) {
    e0 = fmax(e0, __shfl_down_sync(0xffffffffu, e0, o));
    e1 = fmax(e1, __shfl_down_sync(0xffffffffu, e1, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(reinterpret_cast<unsigned long long *>(err), (unsigned long long)__double_as_longlong(e0));
    atomicMax(reinterpret_cast<unsigned long long *>(err) + 1, (unsigned long long)__double_as_longlong(e1));
  }
}

// per-tet records from the FP64 master element data
__global__ void k_build_records(int nT, const int4 *__restrict__ E, const double *__restrict__ dphi9,
                                const double *__restrict__ vol, const double *__restrict__ params,
                                const double *__restrict__ density, TetRec32 *__restrict__ r32,
                                TetRec64 *__restrict__ r64) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nT; t += gridDim.x * blockDim.x) {
    TetRec32 a;
    TetRec64 b;
    a.idx = E[t];
    b.idx = E[t];
    for (int i = 0; i < 9; ++i) {
      b.dphi[i] = dphi9[9ll * t + i];
      a.dphi[i] = (float)b.dphi[i];
    }
    double v = vol[t];
    b.pv[0] = v * params[2ll * t];
    b.pv[1] = v * params[2ll * t + 1];
    b.mass = density[t] * v;
    b.vol = v;
    b.pad = 0.0;
    a.pv[0] = (float)b.pv[0];
    a.pv[1] = (float)b.pv[1];
    a.mass = (float)b.mass;
    r32[t] = a;
    r64[t] = b;
  }
}

// FP32 per-vertex input of the Hessian kernel: displacement from the rest
// shape (consistent element data, F = I + ...) or raw position.
// u = q - X as an unevaluated float pair u = hi + lo (hi the nearest float,
// lo the float nearest to the remainder): the edge differences that form F
// then keep FP32 accuracy relative to themselves, instead of relative to |u|,
// which under large deformation is many elements' length.
__global__ void k_prep_u(int nV, const double *__restrict__ x, const double *__restrict__ q_base, double scale,
                         const double *__restrict__ X, float4 *__restrict__ u, float4 *__restrict__ ul) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nV; v += gridDim.x * blockDim.x) {
    double q[3];
    float hi[3], lo[3];
    for (int d = 0; d < 3; ++d) {
      q[d] = scale * x[3 * v + d];
      if (q_base) q[d] += q_base[3 * v + d];
      if (X) q[d] -= X[3 * v + d];
      hi[d] = (float)q[d];
      lo[d] = (float)(q[d] - (double)hi[d]);
    }
    u[v] = make_float4(hi[0], hi[1], hi[2], 0.f);
    ul[v] = make_float4(lo[0], lo[1], lo[2], 0.f);
  }
}

// ---------------------------------------------------------- FP64 energy -----
// Displacement gradient H = F - I of tet r at positions q = q_base + scale x,
// from FP64 displacements u = q - X when the element data belongs to the rest
// shape X (exact rest: H = 0), else F - I from positions.
__device__ __forceinline__ void disp_grad64(const TetRec64 &r, const double *__restrict__ x,
                                            const double *__restrict__ q_base, double scale,
                                            const double *__restrict__ X, const double *__restrict__ dx,
                                            double alpha, double *H) {
  const int id[4] = {r.idx.x, r.idx.y, r.idx.z, r.idx.w};
  double u[4][3];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const int i = 3 * id[a] + d;
      double xv = x[i];
      if (dx) xv += alpha * dx[i];
      double base = q_base ? q_base[i] : 0.0;
      if (X) base -= X[i];
      u[a][d] = base + scale * xv;
    }
  def_grad(H, u[0], u[1], u[2], u[3], r.dphi, false);
  if (!X) {
    H[0] -= 1.0;
    H[4] -= 1.0;
    H[8] -= 1.0;
  }
}

template <int MODEL>
__global__ void k_energy(int nT, const TetRec64 *__restrict__ rec, const double *__restrict__ x,
                         const double *__restrict__ q_base, double scale, const double *__restrict__ X,
                         double mass_coeff, const double *__restrict__ x_hat, int ndof,
                         const double *__restrict__ f_ext, double force_scale, double *__restrict__ partial) {
  double acc = 0.0;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nT; t += gridDim.x * blockDim.x) {
    const TetRec64 &r = rec[t];
    double H[9];
    disp_grad64(r, x, q_base, scale, X, nullptr, 0.0, H);
    acc += psi_model_disp<double>(MODEL, H, r.pv);
    if (mass_coeff != 0.0) {
      const int id[4] = {r.idx.x, r.idx.y, r.idx.z, r.idx.w};
      double s[3] = {0, 0, 0}, sh[3] = {0, 0, 0}, xx = 0.0, xh = 0.0;
      for (int a = 0; a < 4; ++a)
        for (int d = 0; d < 3; ++d) {
          const double xv = x[3 * id[a] + d];
          const double h = x_hat ? x_hat[3 * id[a] + d] : 0.0;
          s[d] += xv;
          sh[d] += h;
          xx += xv * xv;
          xh += xv * h;
        }
      double m20 = r.mass / 20.0;
      acc += mass_coeff * m20 * (0.5 * (dot3(s, s) + xx) - (dot3(s, sh) + xh));
    }
  }
  if (f_ext && force_scale != 0.0)
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ndof; i += gridDim.x * blockDim.x)
      acc -= force_scale * f_ext[i] * x[i];
  double s = block_sum(acc);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

// Energy of every tet, psi(F) vol at positions q (linear_tet_*_q,
// src/linear_tet_neohookean_q.cpp:5-18): the per-element terms k_energy sums.
template <int MODEL>
__global__ void k_energy_elem(int nT, const TetRec64 *__restrict__ rec, const double *__restrict__ q,
                              const double *__restrict__ X, double *__restrict__ e) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nT; t += gridDim.x * blockDim.x) {
    double H[9];
    disp_grad64(rec[t], q, nullptr, 1.0, X, nullptr, 0.0, H);
    e[t] = psi_model_disp<double>(MODEL, H, rec[t].pv);
  }
}

// f(x + alpha d) - f(x) of the objective, element by element, so that the
// constant part of f (which dominates |f| near a minimum) cancels exactly:
// per tet psi(H1) - psi(H0), alpha d^T M (x - x_hat) + alpha^2/2 d^T M d,
// and - force_scale alpha d^T f.
template <int MODEL>
__global__ void k_energy_diff(int nT, const TetRec64 *__restrict__ rec, const double *__restrict__ x,
                              const double *__restrict__ dx, double alpha, const double *__restrict__ q_base,
                              double scale, const double *__restrict__ X, double mass_coeff,
                              const double *__restrict__ x_hat, int ndof, const double *__restrict__ f_ext,
                              double force_scale, double *__restrict__ partial) {
  double acc = 0.0;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nT; t += gridDim.x * blockDim.x) {
    const TetRec64 &r = rec[t];
    double H0[9], H1[9];
    disp_grad64(r, x, q_base, scale, X, nullptr, 0.0, H0);
    disp_grad64(r, x, q_base, scale, X, dx, alpha, H1);
    acc += psi_model_disp<double>(MODEL, H1, r.pv) - psi_model_disp<double>(MODEL, H0, r.pv);
    if (mass_coeff != 0.0) {
      const int id[4] = {r.idx.x, r.idx.y, r.idx.z, r.idx.w};
      double sd[3] = {0, 0, 0}, se[3] = {0, 0, 0}, de = 0.0, dd = 0.0;
      for (int a = 0; a < 4; ++a)
        for (int d = 0; d < 3; ++d) {
          const int i = 3 * id[a] + d;
          const double dv = dx[i], ev = x[i] - (x_hat ? x_hat[i] : 0.0);
          sd[d] += dv;
          se[d] += ev;
          de += dv * ev;
          dd += dv * dv;
        }
      // d^T M_e y = m/20 (sum d . sum y + sum_a d_a . y_a)
      const double m20 = r.mass / 20.0;
      acc += mass_coeff * m20 * (alpha * (dot3(sd, se) + de) + 0.5 * alpha * alpha * (dot3(sd, sd) + dd));
    }
  }
  if (f_ext && force_scale != 0.0)
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ndof; i += gridDim.x * blockDim.x)
      acc -= force_scale * alpha * f_ext[i] * dx[i];
  double s = block_sum(acc);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

// Packed meshes: the terms of f(x + alpha_s d) - f(x) with every tet and
// vertex taking its own segment's step (tseg / vseg): per tet the elastic and
// mass difference (as k_energy_diff), per vertex the force term. A term whose
// step is 0 is 0. The per-segment sums follow in fixed order.
template <int MODEL>
__global__ void k_energy_diff_seg(int nT, int nV, const TetRec64 *__restrict__ rec, const double *__restrict__ x,
                                  const double *__restrict__ dx, const double *__restrict__ alpha_seg,
                                  const int *__restrict__ tseg, const int *__restrict__ vseg,
                                  const double *__restrict__ q_base, double scale, const double *__restrict__ X,
                                  double mass_coeff, const double *__restrict__ x_hat, const double *__restrict__ f_ext,
                                  double force_scale, double *__restrict__ et, double *__restrict__ ev) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nT; t += gridDim.x * blockDim.x) {
    const double alpha = alpha_seg[tseg[t]];
    if (alpha == 0.0) {
      et[t] = 0.0;
      continue;
    }
    const TetRec64 &r = rec[t];
    double H0[9], H1[9];
    disp_grad64(r, x, q_base, scale, X, nullptr, 0.0, H0);
    disp_grad64(r, x, q_base, scale, X, dx, alpha, H1);
    double acc = psi_model_disp<double>(MODEL, H1, r.pv) - psi_model_disp<double>(MODEL, H0, r.pv);
    if (mass_coeff != 0.0) {
      const int id[4] = {r.idx.x, r.idx.y, r.idx.z, r.idx.w};
      double sd[3] = {0, 0, 0}, se[3] = {0, 0, 0}, de = 0.0, dd = 0.0;
      for (int a = 0; a < 4; ++a)
        for (int d = 0; d < 3; ++d) {
          const int i = 3 * id[a] + d;
          const double dv = dx[i], evv = x[i] - (x_hat ? x_hat[i] : 0.0);
          sd[d] += dv;
          se[d] += evv;
          de += dv * evv;
          dd += dv * dv;
        }
      const double m20 = r.mass / 20.0;
      acc += mass_coeff * m20 * (alpha * (dot3(sd, se) + de) + 0.5 * alpha * alpha * (dot3(sd, sd) + dd));
    }
    et[t] = acc;
  }
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nV; v += gridDim.x * blockDim.x) {
    const double alpha = alpha_seg[vseg[v]];
    double acc = 0.0;
    if (f_ext && force_scale != 0.0 && alpha != 0.0)
      for (int d = 0; d < 3; ++d) acc -= force_scale * alpha * f_ext[3 * v + d] * dx[3 * v + d];
    ev[v] = acc;
  }
}

// deterministic final sum of n partials (one block)
__global__ void k_sum_partials(int n, const double *__restrict__ in, double *__restrict__ out) {
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) acc += in[i];
  double s = block_sum(acc);
  if (threadIdx.x == 0) *out = s;
}

__global__ void k_dot_partials(int n, const double *__restrict__ a, const double *__restrict__ b,
                               double *__restrict__ partial) {
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) acc += a[i] * b[i];
  double s = block_sum(acc);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

// -------------------------------------------------------- FP64 gradient -----
// element gradient (12 doubles per tet, AoS) of the objective
template <int MODEL>
__global__ void k_grad_elem(int nT, const TetRec64 *__restrict__ rec, const double *__restrict__ x,
                            const double *__restrict__ q_base, double scale, double mass_coeff,
                            const double *__restrict__ x_hat, double *__restrict__ ge) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nT; t += gridDim.x * blockDim.x) {
    const TetRec64 &r = rec[t];
    const int id[4] = {r.idx.x, r.idx.y, r.idx.z, r.idx.w};
    double q[4][3], xs[4][3];
    for (int a = 0; a < 4; ++a)
      for (int d = 0; d < 3; ++d) {
        double xv = x[3 * id[a] + d];
        xs[a][d] = xv;
        q[a][d] = scale * xv + (q_base ? q_base[3 * id[a] + d] : 0.0);
      }
    double F[9], P[9], phi[4][3];
    def_grad(F, q[0], q[1], q[2], q[3], r.dphi, false);
    pk1_model<double>(MODEL, F, r.pv, P);
    phi4(r.dphi, phi);
    double out[12];
    for (int a = 0; a < 4; ++a) {
      double g[3];
      mv3(g, P, phi[a]);
      for (int d = 0; d < 3; ++d) out[3 * a + d] = scale * g[d];
    }
    if (mass_coeff != 0.0) {
      double dd[4][3], s[3] = {0, 0, 0};
      for (int a = 0; a < 4; ++a)
        for (int d = 0; d < 3; ++d) {
          dd[a][d] = xs[a][d] - (x_hat ? x_hat[3 * id[a] + d] : 0.0);
          s[d] += dd[a][d];
        }
      double m20 = mass_coeff * r.mass / 20.0;
      for (int a = 0; a < 4; ++a)
        for (int d = 0; d < 3; ++d) out[3 * a + d] += m20 * (s[d] + dd[a][d]);
    }
    double2 *o = reinterpret_cast<double2 *>(ge + 12ll * t);
    for (int i = 0; i < 6; ++i) o[i] = make_double2(out[2 * i], out[2 * i + 1]);
  }
}

// per-vertex sums of element gradients in tet order (src/assemble.cpp:117-128)
__global__ void k_grad_gather(int nV, const int *__restrict__ inc_ptr, const int *__restrict__ inc_tet,
                              const double *__restrict__ ge, const double *__restrict__ f_ext, double force_scale,
                              const unsigned char *__restrict__ pinned, double *__restrict__ g) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nV; v += gridDim.x * blockDim.x) {
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
    const int k1 = inc_ptr[v + 1];
    for (int k = inc_ptr[v]; k < k1; ++k) {
      const int ta = __ldg(inc_tet + k);
      const double *p = ge + 12ll * (ta >> 2) + 3 * (ta & 3);
      s0 += p[0];
      s1 += p[1];
      s2 += p[2];
    }
    if (f_ext && force_scale != 0.0) {
      s0 -= force_scale * f_ext[3 * v];
      s1 -= force_scale * f_ext[3 * v + 1];
      s2 -= force_scale * f_ext[3 * v + 2];
    }
    if (pinned && pinned[v]) s0 = s1 = s2 = 0.0;
    g[3 * v] = s0;
    g[3 * v + 1] = s1;
    g[3 * v + 2] = s2;
  }
}

// ------------------------------------------------- fused FP32 Hessian -------
// One CTA per chunk of consecutive vertices, one thread per vertex. The thread
// walks its incidences in tet order, evaluates the 3x12 slab (row block a) of
// the element Hessian B^T d2psi B vol (PSD-projected if asked), and adds the
// four 3x3 blocks into its CSR rows staged in shared memory at the positions
// precomputed in inc_pos. Every entry is therefore summed over its tets in tet
// order, as the reference's setFromTriplets does. The chunk's values are then
// written out with coalesced stores.
// F of a tet from its vertices' displacement pairs (x = hi, l = lo): the edge
// differences are (hi_a - hi_0) + (lo_a - lo_0).
template <int MODEL>
__device__ __forceinline__ void elem_F_from(const TetRec32 &r, const float4 &x0, const float4 &x1, const float4 &x2,
                                            const float4 &x3, const float4 &l0, const float4 &l1, const float4 &l2,
                                            const float4 &l3, int add_identity, float *F) {
  const float d1[3] = {(x1.x - x0.x) + (l1.x - l0.x), (x1.y - x0.y) + (l1.y - l0.y), (x1.z - x0.z) + (l1.z - l0.z)};
  const float d2[3] = {(x2.x - x0.x) + (l2.x - l0.x), (x2.y - x0.y) + (l2.y - l0.y), (x2.z - x0.z) + (l2.z - l0.z)};
  const float d3[3] = {(x3.x - x0.x) + (l3.x - l0.x), (x3.y - x0.y) + (l3.y - l0.y), (x3.z - x0.z) + (l3.z - l0.z)};
  const float z[3] = {0.f, 0.f, 0.f};
  def_grad(F, z, d1, d2, d3, r.dphi, add_identity != 0);
}

template <int MODEL>
__device__ __forceinline__ void elem_F(const TetRec32 &r, const float4 *__restrict__ u, const float4 *__restrict__ ul,
                                       int add_identity, float *F) {
  elem_F_from<MODEL>(r, __ldg(u + r.idx.x), __ldg(u + r.idx.y), __ldg(u + r.idx.z), __ldg(u + r.idx.w),
                     __ldg(ul + r.idx.x), __ldg(ul + r.idx.y), __ldg(ul + r.idx.z), __ldg(ul + r.idx.w), add_identity,
                     F);
}

template <int MODEL, class Fn>
__device__ __forceinline__ void with_law(const float *F, const float *pv, int corot_exact, Fn &&fn) {
  if constexpr (MODEL == MODEL_NH) fn(LawNH<float>(F, pv));
  else if constexpr (MODEL == MODEL_NH_ISO) fn(LawNHIso<float>(F, pv));
  else if constexpr (MODEL == MODEL_STVK) fn(LawStVK<float>(F, pv));
  else if constexpr (MODEL == MODEL_LE) fn(LawLE<float>(F, pv));
  else if constexpr (MODEL == MODEL_ARAP) {
    float pa[2];
    arap_pv(pv, pa);
    fn(LawCorot<float>(F, pa, corot_exact != 0));
  } else fn(LawCorot<float>(F, pv, corot_exact != 0));
}

// PSD pre-pass, part 1, one thread per tet: decide whether simple_psd_fix
// changes the element matrix beyond its translation modes (the exact test
// psd_fast_ok) and flag the tet; flagged tets are appended to a list (the
// order of the list does not matter: each entry writes only its own tet).
// F and the flag are stored per tet (12 floats) for the assembly kernel.
template <int MODEL>
__global__ void __launch_bounds__(256)
k_psd_test(int nT, const TetRec32 *__restrict__ rec, const float4 *__restrict__ u, const float4 *__restrict__ ul,
           int add_identity, float tol,
           int corot_exact, float4 *__restrict__ fslot, int *__restrict__ list, int *__restrict__ count) {
  for (int t0 = blockIdx.x * blockDim.x; t0 < nT; t0 += gridDim.x * blockDim.x) {
    const int t = t0 + threadIdx.x;
    bool flag = false;
    if (t < nT) {
      TetRec32 r;
      load_rec32(rec, t, r);
      float phi[4][3];
      phi4(r.dphi, phi);
      float F[9];
      elem_F<MODEL>(r, u, ul, add_identity, F);
      with_law<MODEL>(F, r.pv, corot_exact, [&](const auto &law) { flag = !psd_fast_ok(law, phi, tol); });
      // the assembly reads F and the flag from here instead of gathering the vertices again
      float4 *o = fslot + 3ll * t;
      o[0] = make_float4(F[0], F[1], F[2], F[3]);
      o[1] = make_float4(F[4], F[5], F[6], F[7]);
      o[2] = make_float4(F[8], flag ? 1.f : 0.f, 0.f, 0.f);
    }
    // warp-aggregated append
    const unsigned m = __ballot_sync(0xffffffffu, flag);
    if (m) {
      const int lane = threadIdx.x & 31;
      int base = 0;
      if (lane == 0) base = atomicAdd(count, __popc(m));
      base = __shfl_sync(0xffffffffu, base, 0);
      if (flag) list[base + __popc(m & ((1u << lane) - 1u))] = t;
    }
  }
}

// PSD pre-pass, part 2, one thread per flagged tet: the projected 9x9 N
// (packed, 45 floats) of simple_psd_fix.
template <int MODEL>
__global__ void __launch_bounds__(256)
k_psd_eig(const int *__restrict__ list, const int *__restrict__ count, const TetRec32 *__restrict__ rec,
          const float4 *__restrict__ u, const float4 *__restrict__ ul, int add_identity, float tol, int corot_exact,
          float *__restrict__ Nbuf) {
  const int n = *count;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int t = __ldg(list + i);
    TetRec32 r;
    load_rec32(rec, t, r);
    float phi[4][3];
    phi4(r.dphi, phi);
    float F[9];
    elem_F<MODEL>(r, u, ul, add_identity, F);
    with_law<MODEL>(F, r.pv, corot_exact, [&](const auto &law) {
      float N[45];
      psd_eig_N(law, phi, tol, N);
      float *o = Nbuf + 45ll * t;
#pragma unroll
      for (int k = 0; k < 45; ++k) o[k] = N[k];
    });
  }
}

// Inputs of one incidence (tet t seen from its vertex a): the tet record and
// the four vertex positions.
struct HessInc {
  TetRec32 r;
  float4 x[4];
  float4 xl[4];  // lo parts of the vertices' displacement pairs (without the pre-pass)
  uint32_t pos;
  int t, a;
  bool slow;
};

// With the PSD pre-pass (PRE) the tet's F and projection flag come from its
// 12-float slot (x[0..2]) together with the record; otherwise the four vertex
// positions are gathered (x[0..3]) after the record.
template <bool PRE>
__device__ __forceinline__ void load_inc_head(const int *__restrict__ inc_tet, const uint32_t *__restrict__ inc_pos,
                                              const TetRec32 *__restrict__ rec, const float4 *__restrict__ fslot,
                                              int k, HessInc &h) {
  const int ta = __ldg(inc_tet + k);
  h.t = ta >> 2;
  h.a = ta & 3;
  h.pos = __ldg(inc_pos + k);
  load_rec32(rec, ta >> 2, h.r);
  h.slow = false;
  if constexpr (PRE) {
    const float4 *f = fslot + 3ll * h.t;
    h.x[0] = __ldg(f);
    h.x[1] = __ldg(f + 1);
    h.x[2] = __ldg(f + 2);
    h.slow = h.x[2].y != 0.f;
  }
}

template <bool PRE>
__device__ __forceinline__ void load_inc_x(const float4 *__restrict__ u, const float4 *__restrict__ ul, HessInc &h) {
  if constexpr (!PRE) {
    h.x[0] = __ldg(u + h.r.idx.x);
    h.x[1] = __ldg(u + h.r.idx.y);
    h.x[2] = __ldg(u + h.r.idx.z);
    h.x[3] = __ldg(u + h.r.idx.w);
    h.xl[0] = __ldg(ul + h.r.idx.x);
    h.xl[1] = __ldg(ul + h.r.idx.y);
    h.xl[2] = __ldg(ul + h.r.idx.z);
    h.xl[3] = __ldg(ul + h.r.idx.w);
  }
}

// Row block a of one element Hessian: the off-diagonal blocks (b != a) are
// added into the thread's staged CSR rows, the diagonal block (b == a, always
// the thread's own diagonal position) into the registers D.
//
// Unprojected elements: every law is linear in its parameters (K cK =
// K(cK pv)) and bilinear in (pa, pb) with phi_0 = -(phi_1 + phi_2 + phi_3),
// so K_a0 = -(K_a1 + K_a2 + K_a3) and only three blocks are evaluated.
template <int MODEL, bool PSD>
__device__ __forceinline__ void hess_inc(const HessInc &h, float *row, int rs, float *D, int add_identity, float cK,
                                         float cM, float tol, int corot_exact, const float *__restrict__ Nbuf) {
  const int a = h.a;
  float phi[4][3];
  phi4(h.r.dphi, phi);
  float K[4][9];
  if constexpr (MODEL >= 0) {
    if (PSD && h.slow) {
      float N[45];
      const float *src = Nbuf + 45ll * h.t;
#pragma unroll
      for (int i = 0; i < 45; ++i) N[i] = __ldg(src + i);
      psd_blocks_from_N(N, phi, a, K);
#pragma unroll
      for (int b = 0; b < 4; ++b)
#pragma unroll
        for (int i = 0; i < 9; ++i) K[b][i] *= cK;
    } else {
      float F[9];
      if constexpr (PSD) {
        F[0] = h.x[0].x; F[1] = h.x[0].y; F[2] = h.x[0].z; F[3] = h.x[0].w;
        F[4] = h.x[1].x; F[5] = h.x[1].y; F[6] = h.x[1].z; F[7] = h.x[1].w;
        F[8] = h.x[2].x;
      } else {
        elem_F_from<MODEL>(h.r, h.x[0], h.x[1], h.x[2], h.x[3], h.xl[0], h.xl[1], h.xl[2], h.xl[3], add_identity, F);
      }
      const float pv[2] = {cK * h.r.pv[0], cK * h.r.pv[1]};
      float pa[3];
#pragma unroll
      for (int d = 0; d < 3; ++d) pa[d] = a == 0 ? phi[0][d] : a == 1 ? phi[1][d] : a == 2 ? phi[2][d] : phi[3][d];
      with_law<MODEL>(F, pv, corot_exact, [&](const auto &law) {
#pragma unroll
        for (int b = 1; b < 4; ++b) law.block(pa, phi[b], K[b]);
      });
#pragma unroll
      for (int i = 0; i < 9; ++i) K[0][i] = -(K[1][i] + K[2][i] + K[3][i]);
    }
    if constexpr (PSD) {
#pragma unroll
      for (int b = 0; b < 4; ++b) {
        K[b][0] += cK * 0.25f * tol;
        K[b][4] += cK * 0.25f * tol;
        K[b][8] += cK * 0.25f * tol;
      }
    }
  } else {
#pragma unroll
    for (int b = 0; b < 4; ++b)
#pragma unroll
      for (int i = 0; i < 9; ++i) K[b][i] = 0.f;
  }
  if (cM != 0.f) {
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const float m = cM * h.r.mass * (a == b ? 0.1f : 0.05f);
      K[b][0] += m;
      K[b][4] += m;
      K[b][8] += m;
    }
  }
#pragma unroll
  for (int b = 0; b < 4; ++b) {
    if (b == a) {
#pragma unroll
      for (int i = 0; i < 9; ++i) D[i] += K[b][i];
    } else {
      const int j = (h.pos >> (8 * b)) & 255;
#pragma unroll
      for (int kk = 0; kk < 3; ++kk)
#pragma unroll
        for (int ll = 0; ll < 3; ++ll) row[kk * rs + 3 * j + ll] += K[b][3 * kk + ll];
    }
  }
}

// One CTA per chunk of consecutive vertices, one thread per vertex. The thread
// walks its incidences in tet order, evaluates the 3x12 slab (row block a) of
// the element Hessian B^T d2psi B vol (PSD-projected if asked, from the
// pre-pass), and adds the four 3x3 blocks into its CSR rows staged in shared
// memory at the positions precomputed in inc_pos. Every entry is therefore
// summed over its tets in tet order, as the reference's setFromTriplets does.
// Incidences are loaded two at a time (both load chains, incidence -> tet
// record -> vertex positions, in flight together) and added in order. The
// chunk's values are then written out with coalesced stores.
template <int MODEL, bool PSD>
__global__ void __launch_bounds__(kChunkMaxVerts)
k_hess(const int *__restrict__ chunk_v, const int *__restrict__ brp, const int *__restrict__ inc_ptr,
       const int *__restrict__ inc_tet, const uint32_t *__restrict__ inc_pos, const TetRec32 *__restrict__ rec,
       const float4 *__restrict__ u, const float4 *__restrict__ ul, int add_identity, float cK, float cM, float tol,
       int corot_exact, const float4 *__restrict__ fslot, const float *__restrict__ Nbuf, float *__restrict__ values) {
  constexpr bool PRE = PSD && MODEL >= 0;
  extern __shared__ float sbuf[];
  const int v0 = chunk_v[blockIdx.x], v1 = chunk_v[blockIdx.x + 1];
  const int b0 = brp[v0];
  const int len = 9 * (brp[v1] - b0);
  for (int i = threadIdx.x; i < len; i += blockDim.x) sbuf[i] = 0.f;
  __syncthreads();
  const int v = v0 + threadIdx.x;
  if (v < v1) {
    const int rb = brp[v];
    const int rs = 3 * (brp[v + 1] - rb);
    float *row = sbuf + 9 * (rb - b0);
    const int k0 = inc_ptr[v], k1 = inc_ptr[v + 1];
    float D[9];
#pragma unroll
    for (int i = 0; i < 9; ++i) D[i] = 0.f;
    int jd = 0;  // the diagonal block's position in the row
    for (int k = k0; k < k1; k += 2) {
      const bool two = k + 1 < k1;
      HessInc h0, h1;
      load_inc_head<PRE>(inc_tet, inc_pos, rec, fslot, k, h0);
      load_inc_head<PRE>(inc_tet, inc_pos, rec, fslot, two ? k + 1 : k, h1);
      load_inc_x<PRE>(u, ul, h0);
      load_inc_x<PRE>(u, ul, h1);
      jd = (h0.pos >> (8 * h0.a)) & 255;
      hess_inc<MODEL, PSD>(h0, row, rs, D, add_identity, cK, cM, tol, corot_exact, Nbuf);
      if (two) hess_inc<MODEL, PSD>(h1, row, rs, D, add_identity, cK, cM, tol, corot_exact, Nbuf);
    }
    if (k1 > k0) {
#pragma unroll
      for (int kk = 0; kk < 3; ++kk)
#pragma unroll
        for (int ll = 0; ll < 3; ++ll) row[kk * rs + 3 * jd + ll] += D[3 * kk + ll];
    }
  }
  __syncthreads();
  float *out = values + 9ll * b0;
  for (int i = threadIdx.x; i < len; i += blockDim.x) out[i] = sbuf[i];
}

// FP64 mass matrix values in CSR order, with the reference's operations
// (src/linear_tet_mass_matrix.cpp:12-14: mass = density*vol, c0 = (1/10) mass,
// c1 = (1/20) mass) summed per entry in tet order, without FMA contraction.
__global__ void k_mass64(int nV, const int *__restrict__ brp, const int *__restrict__ inc_ptr,
                         const int *__restrict__ inc_tet, const uint32_t *__restrict__ inc_pos,
                         const double *__restrict__ density, const double *__restrict__ vol,
                         double *__restrict__ values) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nV; v += gridDim.x * blockDim.x) {
    const int rb = brp[v], rs = 3 * (brp[v + 1] - rb);
    double *row = values + 9ll * rb;
    for (int i = 0; i < 3 * rs; ++i) row[i] = 0.0;
    for (int k = inc_ptr[v]; k < inc_ptr[v + 1]; ++k) {
      const int ta = inc_tet[k];
      const int t = ta >> 2, a = ta & 3;
      const uint32_t pos = inc_pos[k];
      const double mass = __dmul_rn(density[t], vol[t]);
      const double c0 = __dmul_rn(1.0 / 10.0, mass), c1 = __dmul_rn(1.0 / 20.0, mass);
      for (int b = 0; b < 4; ++b) {
        const int j = (pos >> (8 * b)) & 255;
        const double c = (a == b) ? c0 : c1;
        for (int kk = 0; kk < 3; ++kk)
          for (int ll = 0; ll < 3; ++ll) {
            double *p = row + kk * rs + 3 * j + ll;
            *p = __dadd_rn(*p, kk == ll ? c : 0.0);
          }
      }
    }
  }
}

// assemble (src/assemble.cpp:57-94) of caller-supplied element matrices: Ke
// holds 144 doubles per tet (column-major 12 x 12, row / column 3a + k for
// local vertex a, coordinate k). Each entry of v's rows is summed over its
// tets in tet order from zero, the order in which setFromTriplets sums the
// reference's duplicate triplets, so the FP64 result is the reference's.
__global__ void k_assemble_elem64(int nV, const int *__restrict__ brp, const int *__restrict__ inc_ptr,
                                  const int *__restrict__ inc_tet, const uint32_t *__restrict__ inc_pos,
                                  const double *__restrict__ Ke, double *__restrict__ values) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nV; v += gridDim.x * blockDim.x) {
    const int rb = brp[v], rs = 3 * (brp[v + 1] - rb);
    double *row = values + 9ll * rb;
    for (int i = 0; i < 3 * rs; ++i) row[i] = 0.0;
    for (int k = inc_ptr[v]; k < inc_ptr[v + 1]; ++k) {
      const int ta = inc_tet[k];
      const double *K = Ke + 144ll * (ta >> 2);
      const int a = ta & 3;
      const uint32_t pos = inc_pos[k];
      for (int b = 0; b < 4; ++b) {
        const int j = (pos >> (8 * b)) & 255;
        for (int kk = 0; kk < 3; ++kk)
          for (int ll = 0; ll < 3; ++ll) {
            double *p = row + kk * rs + 3 * j + ll;
            *p = __dadd_rn(*p, K[(3 * a + kk) + 12 * (3 * b + ll)]);
          }
      }
    }
  }
}

// linear_tetmesh_const_ext_force: f_v = sum over tets (tet order) of
// traction * (0.25 vol), as src/linear_tet_const_ext_force.cpp:8-9 + :126.
__global__ void k_force(int nV, const int *__restrict__ inc_ptr, const int *__restrict__ inc_tet,
                        const double *__restrict__ vol, double tx, double ty, double tz, double *__restrict__ f) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nV; v += gridDim.x * blockDim.x) {
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
    for (int k = inc_ptr[v]; k < inc_ptr[v + 1]; ++k) {
      const double w = __dmul_rn(0.25, vol[inc_tet[k] >> 2]);
      s0 = __dadd_rn(s0, __dmul_rn(tx, w));
      s1 = __dadd_rn(s1, __dmul_rn(ty, w));
      s2 = __dadd_rn(s2, __dmul_rn(tz, w));
    }
    f[3 * v] = s0;
    f[3 * v + 1] = s1;
    f[3 * v + 2] = s2;
  }
}

__global__ void k_to_double(int64_t n, const float *__restrict__ a, double *__restrict__ b) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (double)a[i];
}

// scalar CSR pattern of the block pattern: row 3v+k holds the 3 nb_v entries
// of blocks j = 0..nb_v-1, columns 3 bcol + l.
__global__ void k_csr_pattern(int nV, const int *__restrict__ brp, const int *__restrict__ bcol, int *__restrict__ rp,
                              int *__restrict__ col) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nV; v += gridDim.x * blockDim.x) {
    const int rb = brp[v], nb = brp[v + 1] - rb;
    for (int k = 0; k < 3; ++k) rp[3 * v + k] = 9 * rb + 3 * k * nb;
    if (v == nV - 1) rp[3 * nV] = 9 * brp[nV];
    for (int k = 0; k < 3; ++k)
      for (int j = 0; j < nb; ++j)
        for (int l = 0; l < 3; ++l) col[9ll * rb + 3 * k * nb + 3 * j + l] = 3 * bcol[rb + j] + l;
  }
}

// ======================================================== host launchers ====
static inline int grid_for(bartels_ctx ctx, int64_t n, int block) {
  int64_t g = (n + block - 1) / block;
  int64_t cap = (int64_t)ctx->num_sms * 8;
  if (g > cap) g = cap;
  if (g < 1) g = 1;
  return (int)g;
}

int launch_dphi_vol(bartels_ctx ctx, int nV, const double *X3, int nT, const int4 *E, double *dphidX_cm,
                    double *dphi9, double *vol) {
  (void)nV;
  BT_LAUNCH(ctx, k_dphi_vol, grid_for(ctx, nT, 256), 256, 0, nT, X3, E, dphidX_cm, dphi9, vol);
  return BARTELS_OK;
}

int launch_import_dphi(bartels_ctx ctx, bartels_mesh_plan plan, const double *src_d, double *err_d) {
  BT_CUDA(cudaMemsetAsync(err_d, 0, 2 * sizeof(double), ctx->stream));
  BT_LAUNCH(ctx, k_import_dphi, grid_for(ctx, plan->nT, 256), 256, 0, plan->nT, src_d, plan->X, plan->E,
            plan->dphi64, err_d);
  return BARTELS_OK;
}

int plan_refresh_records(bartels_mesh_plan plan) {
  bartels_ctx ctx = plan->ctx;
  BT_LAUNCH(ctx, k_build_records, grid_for(ctx, plan->nT, 256), 256, 0, plan->nT, plan->E, plan->dphi64, plan->vol,
            plan->params, plan->density, plan->rec32, plan->rec64);
  return BARTELS_OK;
}

int launch_prep_u(bartels_ctx ctx, bartels_mesh_plan plan, const double *x, const double *q_base, double scale,
                  bool displacement, float4 *u) {
  BT_LAUNCH(ctx, k_prep_u, grid_for(ctx, plan->nV, 256), 256, 0, plan->nV, x, q_base, scale,
            displacement ? plan->X : (const double *)nullptr, u, u + plan->nV);
  return BARTELS_OK;
}

static constexpr int kRedBlocks = 1024;

int reduce_sum(bartels_ctx ctx, const double *in, int n, double *out) {
  BT_LAUNCH(ctx, k_sum_partials, 1, 1024, 0, n, in, out);
  return BARTELS_OK;
}

int dot(bartels_ctx ctx, const double *a, const double *b, int n, double *out) {
  BT_CHECK(ctx->partials.ensure(kRedBlocks * sizeof(double)));
  const int g = grid_for(ctx, n, 256) < kRedBlocks ? grid_for(ctx, n, 256) : kRedBlocks;
  BT_LAUNCH(ctx, k_dot_partials, g, 256, 0, n, a, b, ctx->partials.as<double>());
  return reduce_sum(ctx, ctx->partials.as<double>(), g, out);
}

int energy_elements(bartels_ctx ctx, bartels_mesh_plan plan, int model, const double *q, double *e) {
  if (plan->nT == 0) return BARTELS_OK;
  const int g = grid_for(ctx, plan->nT, 256);
  const double *X = plan->dphi_matches_rest ? plan->X : nullptr;
#define BT_EE(M) BT_LAUNCH(ctx, k_energy_elem<M>, g, 256, 0, plan->nT, plan->rec64, q, X, e)
  switch (model) {
    case MODEL_NH: BT_EE(MODEL_NH); break;
    case MODEL_STVK: BT_EE(MODEL_STVK); break;
    case MODEL_COROT: BT_EE(MODEL_COROT); break;
    case MODEL_NH_ISO: BT_EE(MODEL_NH_ISO); break;
    case MODEL_ARAP: BT_EE(MODEL_ARAP); break;
    case MODEL_LE: BT_EE(MODEL_LE); break;
    default: return fail(BARTELS_E_INVALID_ARG, "unknown model");
  }
#undef BT_EE
  return BARTELS_OK;
}

int energy(bartels_ctx ctx, bartels_mesh_plan plan, int model, const ObjectiveDev &obj, const double *x,
           double *d_out) {
  BT_CHECK(ctx->partials.ensure(kRedBlocks * sizeof(double)));
  int g = grid_for(ctx, plan->nT, 256);
  if (g > kRedBlocks) g = kRedBlocks;
  double *part = ctx->partials.as<double>();
  const int ndof = 3 * plan->nV;
  const double *X = plan->dphi_matches_rest ? plan->X : nullptr;
#define BT_EN(M)                                                                                                \
  BT_LAUNCH(ctx, k_energy<M>, g, 256, 0, plan->nT, plan->rec64, x, obj.q_base, obj.scale, X, obj.mass_coeff,   \
            obj.x_hat, ndof, obj.f_ext, obj.force_scale, part)
  switch (model) {
    case MODEL_NH: BT_EN(MODEL_NH); break;
    case MODEL_STVK: BT_EN(MODEL_STVK); break;
    case MODEL_COROT: BT_EN(MODEL_COROT); break;
    case MODEL_NH_ISO: BT_EN(MODEL_NH_ISO); break;
    case MODEL_ARAP: BT_EN(MODEL_ARAP); break;
    case MODEL_LE: BT_EN(MODEL_LE); break;
    default: return fail(BARTELS_E_INVALID_ARG, "unknown model");
  }
#undef BT_EN
  return reduce_sum(ctx, part, g, d_out);
}

int energy_diff(bartels_ctx ctx, bartels_mesh_plan plan, int model, const ObjectiveDev &obj, const double *x,
                const double *dx, double alpha, double *d_out) {
  BT_CHECK(ctx->partials.ensure(kRedBlocks * sizeof(double)));
  int g = grid_for(ctx, plan->nT, 256);
  if (g > kRedBlocks) g = kRedBlocks;
  double *part = ctx->partials.as<double>();
  const int ndof = 3 * plan->nV;
  const double *X = plan->dphi_matches_rest ? plan->X : nullptr;
#define BT_ED(M)                                                                                                \
  BT_LAUNCH(ctx, k_energy_diff<M>, g, 256, 0, plan->nT, plan->rec64, x, dx, alpha, obj.q_base, obj.scale, X,    \
            obj.mass_coeff, obj.x_hat, ndof, obj.f_ext, obj.force_scale, part)
  switch (model) {
    case MODEL_NH: BT_ED(MODEL_NH); break;
    case MODEL_STVK: BT_ED(MODEL_STVK); break;
    case MODEL_COROT: BT_ED(MODEL_COROT); break;
    case MODEL_NH_ISO: BT_ED(MODEL_NH_ISO); break;
    case MODEL_ARAP: BT_ED(MODEL_ARAP); break;
    case MODEL_LE: BT_ED(MODEL_LE); break;
    default: return fail(BARTELS_E_INVALID_ARG, "unknown model");
  }
#undef BT_ED
  return reduce_sum(ctx, part, g, d_out);
}

int energy_diff_seg(bartels_ctx ctx, bartels_mesh_plan plan, int model, const ObjectiveDev &obj, const double *x,
                    const double *dx, const double *alpha_seg, const int *tseg, const int *vseg, double *et,
                    double *ev) {
  const int g = grid_for(ctx, std::max(plan->nT, plan->nV), 256);
  const double *X = plan->dphi_matches_rest ? plan->X : nullptr;
#define BT_EDS(M)                                                                                                 \
  BT_LAUNCH(ctx, k_energy_diff_seg<M>, g, 256, 0, plan->nT, plan->nV, plan->rec64, x, dx, alpha_seg, tseg, vseg, \
            obj.q_base, obj.scale, X, obj.mass_coeff, obj.x_hat, obj.f_ext, obj.force_scale, et, ev)
  switch (model) {
    case MODEL_NH: BT_EDS(MODEL_NH); break;
    case MODEL_STVK: BT_EDS(MODEL_STVK); break;
    case MODEL_COROT: BT_EDS(MODEL_COROT); break;
    case MODEL_NH_ISO: BT_EDS(MODEL_NH_ISO); break;
    case MODEL_ARAP: BT_EDS(MODEL_ARAP); break;
    case MODEL_LE: BT_EDS(MODEL_LE); break;
    default: return fail(BARTELS_E_INVALID_ARG, "unknown model");
  }
#undef BT_EDS
  return BARTELS_OK;
}

int gradient(bartels_ctx ctx, bartels_mesh_plan plan, int model, const ObjectiveDev &obj, const double *x,
             double *g) {
  BT_CHECK(plan->w_grad_e.ensure(sizeof(double) * 12 * (size_t)plan->nT));
  double *ge = plan->w_grad_e.as<double>();
  const int gt = grid_for(ctx, plan->nT, 256);
#define BT_GE(M) \
  BT_LAUNCH(ctx, k_grad_elem<M>, gt, 256, 0, plan->nT, plan->rec64, x, obj.q_base, obj.scale, obj.mass_coeff, obj.x_hat, ge)
  switch (model) {
    case MODEL_NH: BT_GE(MODEL_NH); break;
    case MODEL_STVK: BT_GE(MODEL_STVK); break;
    case MODEL_COROT: BT_GE(MODEL_COROT); break;
    case MODEL_NH_ISO: BT_GE(MODEL_NH_ISO); break;
    case MODEL_ARAP: BT_GE(MODEL_ARAP); break;
    case MODEL_LE: BT_GE(MODEL_LE); break;
    default: return fail(BARTELS_E_INVALID_ARG, "unknown model");
  }
#undef BT_GE
  BT_LAUNCH(ctx, k_grad_gather, grid_for(ctx, plan->nV, 256), 256, 0, plan->nV, plan->inc_ptr, plan->inc_tet, ge,
            obj.f_ext, obj.force_scale, obj.pinned, g);
  return BARTELS_OK;
}

template <int MODEL, bool PSD>
static int launch_hess_t(bartels_ctx ctx, bartels_mesh_plan plan, const float4 *u, int add_identity, float cK,
                         float cM, float tol, int corot_exact, float *values) {
  const bool small = plan->hess_chunk == 64 && plan->chunk_v64;
  const int smem = (small ? kChunkFloats / 2 : kChunkFloats) * (int)sizeof(float);
  static bool attr_set = false;  // per template instance
  if (!attr_set) {
    BT_CUDA(cudaFuncSetAttribute(k_hess<MODEL, PSD>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 kChunkFloats * (int)sizeof(float)));
    attr_set = true;
  }
  const int pb = plan->psd_block;
  float4 *fslot = nullptr;
  float *nbuf = nullptr;
  const float4 *ul = u + plan->nV;  // lo parts of the displacement pairs follow the hi parts
  if constexpr (PSD && MODEL >= 0) {
    const size_t nT = (size_t)plan->nT;
    // F + flag slots (12 floats per tet), N (45 floats per tet), the slow-tet list and its count
    BT_CHECK(plan->w_psd.ensure(nT * (57 * sizeof(float) + sizeof(int)) + 512));
    fslot = plan->w_psd.as<float4>();
    nbuf = reinterpret_cast<float *>(fslot + 3 * nT);
    int *list = reinterpret_cast<int *>(nbuf + 45 * nT);
    int *count = list + nT;
    BT_CUDA(cudaMemsetAsync(count, 0, sizeof(int), ctx->stream));
    BT_LAUNCH(ctx, k_psd_test<MODEL>, grid_for(ctx, plan->nT, pb), pb, 0, plan->nT, plan->rec32, u, ul,
              add_identity, tol, corot_exact, fslot, list, count);
    BT_LAUNCH(ctx, k_psd_eig<MODEL>, grid_for(ctx, plan->nT, pb), pb, 0, list, count, plan->rec32, u, ul,
              add_identity, tol, corot_exact, nbuf);
  }
  BT_LAUNCH(ctx, (k_hess<MODEL, PSD>), small ? plan->nchunks64 : plan->nchunks, small ? 64 : kChunkMaxVerts, smem,
            small ? plan->chunk_v64 : plan->chunk_v, plan->brp, plan->inc_ptr, plan->inc_tet, plan->inc_pos,
            plan->rec32, u, ul, add_identity, cK, cM, tol, corot_exact, fslot, nbuf, values);
  return BARTELS_OK;
}

int launch_hess(bartels_ctx ctx, bartels_mesh_plan plan, int model, int psd_mode, const float4 *u, int add_identity,
                float cK, float cM, float tol, int flags, float *values) {
  const int ce = (flags & BARTELS_DQ2_COROT_EXACT) ? 1 : 0;
  const bool psd = psd_mode == BARTELS_PSD_SIMPLE_FIX;
#define BT_H(M)                                                                                  \
  return psd ? launch_hess_t<M, true>(ctx, plan, u, add_identity, cK, cM, tol, ce, values)     \
             : launch_hess_t<M, false>(ctx, plan, u, add_identity, cK, cM, tol, ce, values)
  switch (model) {
    case MODEL_NH: BT_H(MODEL_NH);
    case MODEL_STVK: BT_H(MODEL_STVK);
    case MODEL_COROT: BT_H(MODEL_COROT);
    case MODEL_NH_ISO: BT_H(MODEL_NH_ISO);
    case MODEL_ARAP: BT_H(MODEL_ARAP);
    case MODEL_LE: BT_H(MODEL_LE);
    case -1: return launch_hess_t<-1, false>(ctx, plan, u, add_identity, 0.f, cM, 0.f, 0, values);
    default: return fail(BARTELS_E_INVALID_ARG, "unknown model");
  }
#undef BT_H
}

int launch_mass64(bartels_ctx ctx, bartels_mesh_plan plan, const double *density, const double *vol,
                  double *values) {
  BT_LAUNCH(ctx, k_mass64, grid_for(ctx, plan->nV, 128), 128, 0, plan->nV, plan->brp, plan->inc_ptr, plan->inc_tet,
            plan->inc_pos, density, vol, values);
  return BARTELS_OK;
}

int assemble_elements64(bartels_ctx ctx, bartels_mesh_plan plan, const double *Ke, double *values) {
  BT_LAUNCH(ctx, k_assemble_elem64, grid_for(ctx, plan->nV, 128), 128, 0, plan->nV, plan->brp, plan->inc_ptr,
            plan->inc_tet, plan->inc_pos, Ke, values);
  return BARTELS_OK;
}

// vector assemble (src/assemble.cpp:100-132): per-tet 12-vectors ge (entry
// 3a + k) summed per vertex in tet order
int assemble_vector64(bartels_ctx ctx, bartels_mesh_plan plan, const double *ge, double *g) {
  BT_LAUNCH(ctx, k_grad_gather, grid_for(ctx, plan->nV, 256), 256, 0, plan->nV, plan->inc_ptr, plan->inc_tet, ge,
            nullptr, 0.0, nullptr, g);
  return BARTELS_OK;
}

int ext_force(bartels_ctx ctx, bartels_mesh_plan plan, const double traction[3], double *f) {
  BT_LAUNCH(ctx, k_force, grid_for(ctx, plan->nV, 256), 256, 0, plan->nV, plan->inc_ptr, plan->inc_tet, plan->vol,
            traction[0], traction[1], traction[2], f);
  return BARTELS_OK;
}

int values_to_double(bartels_ctx ctx, const float *v32, double *v64, int64_t n) {
  BT_LAUNCH(ctx, k_to_double, grid_for(ctx, n, 256), 256, 0, n, v32, v64);
  return BARTELS_OK;
}

// ------------------------------------------------ allocation-free gradient ---
// Scratch of bartels_tetmesh_dq_noalloc_d: the 12 per-tet gradient entries of
// up to kNoAllocMaxTets tets (6 MiB). Every GPU that loads the library keeps
// this array until the process exits. All calls share it and it keeps the last
// call's contents; every entry a call reads is written by that call first, so
// nothing needs clearing. Calls that overlap on the GPU race on it.
constexpr int kNoAllocMaxTets = 1 << 16;
static __device__ __align__(256) double g_noalloc_scratch[12 * kNoAllocMaxTets];
// Device address of the scratch, looked up once per device and kept for the
// life of the process. A cudaDeviceReset (or any reset of the device's primary
// context) invalidates it: a process that resets a device must not call the
// allocation-free entry point on that device afterwards.
static double *g_noalloc_ptr[64];
static std::mutex g_noalloc_mutex;

int noalloc_gradient(bartels_ctx ctx, bartels_mesh_plan plan, int model, const double *q_d, double *g_d) {
  if (plan->nT > kNoAllocMaxTets)
    return fail(BARTELS_E_UNSUPPORTED, "bartels_tetmesh_dq_noalloc_d handles at most 65536 tets (the mesh has " +
                                           std::to_string(plan->nT) + "); use bartels_tetmesh_dq");
  if (ctx->device < 0 || ctx->device >= 64) return fail(BARTELS_E_UNSUPPORTED, "device index above 63");
  double *ge;
  {
    // one-time set-up per device (the caller's device is current): the array's
    // host-side name is not a device address, so look the address up
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[ctx->device]) {
      void *p = nullptr;
      BT_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
      g_noalloc_ptr[ctx->device] = static_cast<double *>(p);
    }
    ge = g_noalloc_ptr[ctx->device];
  }
  if (plan->nT == 0) return BARTELS_OK;
  const int gt = grid_for(ctx, plan->nT, 256);
#define BT_GN(M) BT_LAUNCH(ctx, k_grad_elem<M>, gt, 256, 0, plan->nT, plan->rec64, q_d, nullptr, 1.0, 0.0, nullptr, ge)
  switch (model) {
    case MODEL_NH: BT_GN(MODEL_NH); break;
    case MODEL_STVK: BT_GN(MODEL_STVK); break;
    case MODEL_COROT: BT_GN(MODEL_COROT); break;
    case MODEL_NH_ISO: BT_GN(MODEL_NH_ISO); break;
    case MODEL_ARAP: BT_GN(MODEL_ARAP); break;
    case MODEL_LE: BT_GN(MODEL_LE); break;
    default: return fail(BARTELS_E_INVALID_ARG, "unknown model");
  }
#undef BT_GN
  BT_LAUNCH(ctx, k_grad_gather, grid_for(ctx, plan->nV, 256), 256, 0, plan->nV, plan->inc_ptr, plan->inc_tet, ge,
            (const double *)nullptr, 0.0, (const unsigned char *)nullptr, g_d);
  return BARTELS_OK;
}

int plan_build_csr_pattern(bartels_mesh_plan plan) {
  if (plan->csr_rp) return BARTELS_OK;
  bartels_ctx ctx = plan->ctx;
  BT_CUDA(cudaMalloc(&plan->csr_rp, sizeof(int) * (3 * (size_t)plan->nV + 1)));
  BT_CUDA(cudaMalloc(&plan->csr_col, sizeof(int) * 9 * (size_t)plan->nnzb));
  BT_LAUNCH(ctx, k_csr_pattern, grid_for(ctx, plan->nV, 128), 128, 0, plan->nV, plan->brp, plan->bcol, plan->csr_rp,
            plan->csr_col);
  return BARTELS_OK;
}

}  // namespace bartels
