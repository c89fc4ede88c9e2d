// Triangle meshes. In the plane (linear_tri2dmesh_* of the reference): per-element
// energy, gradient and Hessian of every material law, mass matrix; in space
// (linear_tri3dmesh_*): shape gradients and the StVK membrane Hessian. Both
// assemble deterministically into a CSR whose pattern (dim x dim vertex blocks,
// rows dim v .. dim v + dim - 1 with the sorted columns of v's neighbours) is
// the reference's.
//
// The reference embeds the 2D deformation gradient in 3D (F33 = 1, the other
// out-of-plane entries 0) and restricts B^T d2psi B to the in-plane DOFs
// (src/linear_tri2d_neohookean_dq2.cpp:9-31 and the other linear_tri2d_* files).
// Here the same 3D laws are evaluated at that F: the 2x2 block of nodes a, b is
// the top-left of the 3D block law.block(pa, pb) with pa = (dphi_a/dX, 0), the
// gradient is P (the 3D first Piola-Kirchhoff stress) contracted with pa, and
// every law is linear in its parameters, so the element area scales them.
//
// 2D meshes are small next to the tet workloads, so everything here is FP64:
// energies, gradients, Hessians and the simple_psd_fix eigen-solve (6x6 cyclic
// Jacobi, eigenvalues below tol raised to tol, as src/simple_psd_fix.cpp:9-19).
#include "internal.cuh"
#include "devmath.cuh"

#include <algorithm>
#include <cmath>
#include <vector>

struct bartels_tri_plan_s {
  bartels_ctx ctx = nullptr;
  int nV = 0, nT = 0;
  int dim = 2;                   // DOFs per vertex: 2 (planar meshes) or 3 (triangles in space)
  int64_t nnzb = 0;
  int4 *E = nullptr;             // nT (x, y, z used)
  int *brp = nullptr, *bcol = nullptr;
  int *inc_ptr = nullptr, *inc = nullptr;  // per vertex: (tri << 2 | local index), tris ascending
  uint32_t *inc_pos = nullptr;   // per incidence: positions of the tri's 3 vertices in the row (8 bits each)
  std::vector<int> h_brp, h_bcol;
  bartels::DevBuf w_in, w_elem, w_out;
};

namespace bartels {
namespace {

// src/linear_tri2d_dphi_dX.cpp:10-16: rows 1, 2 of dphi = inverse of the edge
// matrix [x1 - x0, x2 - x0] (inverse22, include/EigenTypes.h:122-130), row 0 =
// minus their sum; stored as the column-major flatten of the 3x2 matrix.
__global__ void k_tri2d_dphi(int nV, int nT, const double *__restrict__ V, const int4 *__restrict__ E,
                             double *__restrict__ dphi, double *__restrict__ area) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nT; t += gridDim.x * blockDim.x) {
    const int4 e = E[t];
    const double x0 = V[e.x], y0 = V[e.x + nV];
    const double a00 = V[e.y] - x0, a10 = V[e.y + nV] - y0;  // column 0: x1 - x0
    const double a01 = V[e.z] - x0, a11 = V[e.z + nV] - y0;  // column 1: x2 - x0
    const double det = a00 * a11 - a01 * a10;
    const double inv = 1.0 / det;
    const double i00 = a11 * inv, i10 = -a10 * inv, i01 = -a01 * inv, i11 = a00 * inv;
    // dphi(a, c) at t + nT (a + 3 c)
    dphi[t + (size_t)nT * 1] = i00;
    dphi[t + (size_t)nT * 4] = i01;
    dphi[t + (size_t)nT * 2] = i10;
    dphi[t + (size_t)nT * 5] = i11;
    dphi[t + (size_t)nT * 0] = -(i00 + i10);
    dphi[t + (size_t)nT * 3] = -(i01 + i11);
    if (area) area[t] = 0.5 * fabs(det);
  }
}

struct TriElem {
  double F[9];      // embedded deformation gradient, column-major
  double phi[3][3]; // (dphi_a/dX, dphi_a/dY, 0)
  double pv[2];     // area * params
};

__device__ __forceinline__ void tri_load(int t, int nT, const int4 *__restrict__ E, const double *__restrict__ q,
                                         const double *__restrict__ dphi, const double *__restrict__ area,
                                         const double *__restrict__ params, TriElem &el) {
  const int4 e = E[t];
  const int id[3] = {e.x, e.y, e.z};
  for (int a = 0; a < 3; ++a) {
    el.phi[a][0] = dphi[t + (size_t)nT * a];
    el.phi[a][1] = dphi[t + (size_t)nT * (a + 3)];
    el.phi[a][2] = 0.0;
  }
  for (int i = 0; i < 9; ++i) el.F[i] = 0.0;
  for (int k = 0; k < 2; ++k)
    for (int i = 0; i < 2; ++i) {
      double s = 0.0;
      for (int a = 0; a < 3; ++a) s += q[2 * id[a] + k] * el.phi[a][i];
      el.F[k + 3 * i] = s;
    }
  el.F[8] = 1.0;
  const double A = area[t];
  el.pv[0] = A * params[t];
  el.pv[1] = A * params[t + (size_t)nT];
}

// Symmetric N x N (row-major, in place) -> W max(L, tol) W^T: cyclic Jacobi
// until the off-diagonal mass is at rounding level (at most 40 sweeps).
template <int N>
__device__ void psd_fix_n(double *A, double tol) {
  double W[N * N];
  for (int i = 0; i < N * N; ++i) W[i] = (i % (N + 1) == 0) ? 1.0 : 0.0;
  for (int s = 0; s < 40; ++s) {
    double off = 0.0, dia = 0.0;
    for (int i = 0; i < N; ++i) {
      dia += A[(N + 1) * i] * A[(N + 1) * i];
      for (int j = 0; j < i; ++j) off += A[N * i + j] * A[N * i + j];
    }
    if (off <= 1e-32 * dia) break;
    for (int p = 0; p < N - 1; ++p)
      for (int r = p + 1; r < N; ++r) {
        const double apr = A[N * p + r];
        if (apr == 0.0) continue;
        const double theta = (A[N * r + r] - A[N * p + p]) / (2.0 * apr);
        const double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        const double c = 1.0 / sqrt(t * t + 1.0), sn = t * c;
        for (int k = 0; k < N; ++k) {  // columns p, r
          const double akp = A[N * k + p], akr = A[N * k + r];
          A[N * k + p] = c * akp - sn * akr;
          A[N * k + r] = sn * akp + c * akr;
        }
        for (int k = 0; k < N; ++k) {  // rows p, r
          const double apk = A[N * p + k], ark = A[N * r + k];
          A[N * p + k] = c * apk - sn * ark;
          A[N * r + k] = sn * apk + c * ark;
        }
        for (int k = 0; k < N; ++k) {
          const double wkp = W[N * k + p], wkr = W[N * k + r];
          W[N * k + p] = c * wkp - sn * wkr;
          W[N * k + r] = sn * wkp + c * wkr;
        }
      }
  }
  double L[N];
  for (int i = 0; i < N; ++i) L[i] = A[(N + 1) * i] < tol ? tol : A[(N + 1) * i];
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) {
      double s = 0.0;
      for (int k = 0; k < N; ++k) s += W[N * i + k] * L[k] * W[N * j + k];
      A[N * i + j] = s;
    }
}

// what: 0 energy (1 per tri), 1 gradient (6), 2 Hessian (36, row-major, DOF 2a + k)
__global__ void k_tri2d_elem(int what, int model, int nT, const int4 *__restrict__ E, const double *__restrict__ q,
                             const double *__restrict__ dphi, const double *__restrict__ area,
                             const double *__restrict__ params, int psd, double tol, double *__restrict__ out) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nT; t += gridDim.x * blockDim.x) {
    TriElem el;
    tri_load(t, nT, E, q, dphi, area, params, el);
    if (what == 0) {
      out[t] = psi_model<double>(model, el.F, el.pv);
    } else if (what == 1) {
      double P[9];
      pk1_model<double>(model, el.F, el.pv, P);
      for (int a = 0; a < 3; ++a)
        for (int k = 0; k < 2; ++k) out[6ll * t + 2 * a + k] = P[k] * el.phi[a][0] + P[k + 3] * el.phi[a][1];
    } else {
      double K[36];
      with_law64(model, el.F, el.pv, [&](const auto &law) {
        for (int a = 0; a < 3; ++a)
          for (int b = 0; b < 3; ++b) {
            double B3[9];
            law.block(el.phi[a], el.phi[b], B3);
            for (int k = 0; k < 2; ++k)
              for (int l = 0; l < 2; ++l) K[6 * (2 * a + k) + 2 * b + l] = B3[3 * k + l];
          }
      });
      if (psd) psd_fix_n<6>(K, tol);
      for (int i = 0; i < 36; ++i) out[36ll * t + i] = K[i];
    }
  }
}

// consistent mass (src/linear_tri2d_mass_matrix.cpp:10-32): density * area *
// (1/6 on the diagonal blocks, 1/12 off) x I2
__global__ void k_tri2d_mass(int nT, const double *__restrict__ density, const double *__restrict__ area,
                             double *__restrict__ out) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nT; t += gridDim.x * blockDim.x) {
    const double mass = density[t] * area[t];
    const double c0 = (1.0 / 6.0) * mass, c1 = (1.0 / 12.0) * mass;
    for (int i = 0; i < 36; ++i) {
      const int r = i / 6, c = i % 6;
      out[36ll * t + i] = (r % 2 != c % 2) ? 0.0 : (r / 2 == c / 2 ? c0 : c1);
    }
  }
}

// per-vertex sums in tri order (src/assemble.cpp:100-132)
__global__ void k_tri2d_gather_vec(int nV, const int *__restrict__ inc_ptr, const int *__restrict__ inc,
                                   const double *__restrict__ ge, double *__restrict__ g) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nV; v += gridDim.x * blockDim.x) {
    double s0 = 0.0, s1 = 0.0;
    for (int k = inc_ptr[v]; k < inc_ptr[v + 1]; ++k) {
      const int ta = inc[k], t = ta >> 2, a = ta & 3;
      s0 += ge[6ll * t + 2 * a];
      s1 += ge[6ll * t + 2 * a + 1];
    }
    g[2 * v] = s0;
    g[2 * v + 1] = s1;
  }
}

// Rows D v .. D v + D - 1 of the CSR: every entry summed over the vertex's tris
// in tri order (as setFromTriplets sums duplicates, src/assemble.cpp:57-94),
// from element matrices of 3D x 3D (row-major, DOF D a + k). The thread owns
// its rows' segment [D^2 brp[v], D^2 brp[v + 1]) of the values.
template <int D>
__global__ void k_tri_gather_mat(int nV, const int *__restrict__ brp, const int *__restrict__ inc_ptr,
                                 const int *__restrict__ inc, const uint32_t *__restrict__ inc_pos,
                                 const double *__restrict__ ke, double *__restrict__ vals) {
  constexpr int NE = 3 * D;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nV; v += gridDim.x * blockDim.x) {
    const int rb = brp[v], rs = D * (brp[v + 1] - rb);
    double *row = vals + (long long)D * D * rb;
    for (int i = 0; i < D * rs; ++i) row[i] = 0.0;
    for (int k = inc_ptr[v]; k < inc_ptr[v + 1]; ++k) {
      const int ta = inc[k], t = ta >> 2, a = ta & 3;
      const uint32_t pos = inc_pos[k];
      const double *K = ke + (long long)NE * NE * t;
      for (int b = 0; b < 3; ++b) {
        const int j = (pos >> (8 * b)) & 255;
        for (int kk = 0; kk < D; ++kk)
          for (int ll = 0; ll < D; ++ll) row[kk * rs + D * j + ll] += K[NE * (D * a + kk) + D * b + ll];
      }
    }
  }
}

// src/linear_tri3d_dphi_dX.cpp:10-16: with T = [x1 - x0, x2 - x0] (3x2), rows
// 1, 2 of dphi = (T^T T)^-1 T^T and row 0 = minus their sum; stored as the
// column-major flatten of the 3x3 matrix. area = |e1 x e2| / 2.
__global__ void k_tri3d_dphi(int nV, int nT, const double *__restrict__ V, const int4 *__restrict__ E,
                             double *__restrict__ dphi, double *__restrict__ area) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nT; t += gridDim.x * blockDim.x) {
    const int4 e = E[t];
    double e1[3], e2[3];
    for (int c = 0; c < 3; ++c) {
      e1[c] = V[e.y + (size_t)nV * c] - V[e.x + (size_t)nV * c];
      e2[c] = V[e.z + (size_t)nV * c] - V[e.x + (size_t)nV * c];
    }
    const double g11 = e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2];
    const double g12 = e1[0] * e2[0] + e1[1] * e2[1] + e1[2] * e2[2];
    const double g22 = e2[0] * e2[0] + e2[1] * e2[1] + e2[2] * e2[2];
    const double det = g11 * g22 - g12 * g12, inv = 1.0 / det;
    for (int c = 0; c < 3; ++c) {
      const double r1 = (g22 * e1[c] - g12 * e2[c]) * inv;  // row 1 of (T^T T)^-1 T^T
      const double r2 = (-g12 * e1[c] + g11 * e2[c]) * inv;  // row 2
      dphi[t + (size_t)nT * (1 + 3 * c)] = r1;
      dphi[t + (size_t)nT * (2 + 3 * c)] = r2;
      dphi[t + (size_t)nT * (3 * c)] = -(r1 + r2);
    }
    if (area) area[t] = 0.5 * sqrt(det);
  }
}

// StVK d2psi/dF2 (9x9, rows (k, i) -> k + 3 i, columns (l, j) -> l + 3 j):
// H = delta_kl S_ij + mu (F F^T)_kl delta_ij + mu F_kj F_li + lambda F_ki F_lj,
// S = 2 mu E + lambda tr(E) I, E = (F^T F - I) / 2 (src/d2psi_stvk_dF2.cpp).
__device__ void stvk_h9(const double *F, double lam, double mu, double *H) {
  double C[9], S[9], FF[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double c = 0.0, f = 0.0;
      for (int k = 0; k < 3; ++k) {
        c += F[k + 3 * i] * F[k + 3 * j];
        f += F[i + 3 * k] * F[j + 3 * k];
      }
      C[i + 3 * j] = c;
      FF[i + 3 * j] = f;
    }
  const double trE = 0.5 * (C[0] + C[4] + C[8] - 3.0);
  for (int i = 0; i < 9; ++i) S[i] = mu * (C[i] - ((i % 4) == 0 ? 1.0 : 0.0)) + ((i % 4) == 0 ? lam * trE : 0.0);
  for (int k = 0; k < 3; ++k)
    for (int i = 0; i < 3; ++i)
      for (int l = 0; l < 3; ++l)
        for (int j = 0; j < 3; ++j) {
          double h = mu * F[k + 3 * j] * F[l + 3 * i] + lam * F[k + 3 * i] * F[l + 3 * j];
          if (k == l) h += S[i + 3 * j];
          if (i == j) h += mu * FF[k + 3 * l];
          H[9 * (k + 3 * i) + (l + 3 * j)] = h;
        }
}

// src/linear_tri3d_stvk_dq2.cpp:15-42: B = flatten_multiply_right(dphidX) +
// flatten_multiply_right(N) unflatten<3,9>(dndq), F = unflatten(B qe + vec(n N^T)),
// element Hessian B^T d2psi(F) B * area (9x9 row-major, DOF 3a + k), with the
// optional simple_psd_fix; the caller supplies the rest normal N, the deformed
// normal n and its derivative dn/dqe per element.
__global__ void k_tri3d_stvk_hess(int nT, const int4 *__restrict__ E, const double *__restrict__ q,
                                  const double *__restrict__ dphi, const double *__restrict__ Nr,
                                  const double *__restrict__ nd, const double *__restrict__ dndq,
                                  const double *__restrict__ area, const double *__restrict__ params, int psd,
                                  double tol, double *__restrict__ out) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nT; t += gridDim.x * blockDim.x) {
    const int4 e = E[t];
    const int id[3] = {e.x, e.y, e.z};
    double qe[9], M[9], N[3], n[3], B[81], F[9];
    for (int a = 0; a < 3; ++a)
      for (int k = 0; k < 3; ++k) qe[3 * a + k] = q[3 * id[a] + k];
    for (int i = 0; i < 9; ++i) M[i] = dphi[t + (size_t)nT * i];  // M(a, c) at a + 3 c
    for (int c = 0; c < 3; ++c) {
      N[c] = Nr[t + (size_t)nT * c];
      n[c] = nd[t + (size_t)nT * c];
    }
    // B(k + 3 i, 3 a + l) = delta_kl M(a, i) + N_i dndq(k, 3 a + l)
    for (int k = 0; k < 3; ++k)
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 9; ++j) {
          const int a = j / 3, l = j % 3;
          B[9 * (k + 3 * i) + j] = (k == l ? M[a + 3 * i] : 0.0) + N[i] * dndq[t + (size_t)nT * (k + 3 * j)];
        }
    for (int r = 0; r < 9; ++r) {
      double s = n[r % 3] * N[r / 3];
      for (int j = 0; j < 9; ++j) s += B[9 * r + j] * qe[j];
      F[r] = s;
    }
    double H[81], HB[81];
    stvk_h9(F, params[t], params[t + (size_t)nT], H);
    for (int r = 0; r < 9; ++r)
      for (int j = 0; j < 9; ++j) {
        double s = 0.0;
        for (int m = 0; m < 9; ++m) s += H[9 * r + m] * B[9 * m + j];
        HB[9 * r + j] = s;
      }
    const double A = area[t];
    double K[81];
    for (int i = 0; i < 9; ++i)
      for (int j = 0; j < 9; ++j) {
        double s = 0.0;
        for (int r = 0; r < 9; ++r) s += B[9 * r + i] * HB[9 * r + j];
        K[9 * i + j] = s * A;
      }
    if (psd) psd_fix_n<9>(K, tol);
    for (int i = 0; i < 81; ++i) out[81ll * t + i] = K[i];
  }
}

template <class T>
int tri_upload(bartels_ctx ctx, T **dst, const T *src, size_t n) {
  BT_CUDA(cudaMalloc(dst, sizeof(T) * std::max<size_t>(n, 1)));
  if (n) BT_CUDA(cudaMemcpyAsync(*dst, src, sizeof(T) * n, cudaMemcpyHostToDevice, ctx->stream));
  return BARTELS_OK;
}

int grid1(bartels_ctx ctx, int64_t n) {
  int64_t g = (n + 255) / 256, cap = (int64_t)ctx->num_sms * 8;
  return (int)std::max<int64_t>(1, std::min(g, cap));
}

int check_tri(bartels_ctx ctx, bartels_tri_plan p, int dim) {
  if (!ctx || !p) return fail(BARTELS_E_INVALID_ARG, "null context or plan");
  if (p->ctx != ctx) return fail(BARTELS_E_INVALID_ARG, "plan belongs to another context");
  if (p->dim != dim) return fail(BARTELS_E_INVALID_ARG, "plan has the wrong number of DOFs per vertex");
  BT_CUDA(cudaSetDevice(ctx->device));
  return BARTELS_OK;
}

// Linear elasticity takes (Young's modulus, Poisson ratio) per element
// (src/d2psi_linear_elasticity_de2.cpp:10-11); the laws take (lambda, mu).
void tri_params(int model, const double *params, int nT, std::vector<double> &buf) {
  buf.assign(params, params + 2 * (size_t)nT);
  if (model != BARTELS_LINEAR_ELASTICITY) return;
  for (int t = 0; t < nT; ++t) {
    const double E = params[t], nu = params[t + (size_t)nT];
    buf[t] = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
    buf[t + (size_t)nT] = E / (2.0 * (1.0 + nu));
  }
}

// upload q (2 nV), dphidX (6 nT), area (nT), params (2 nT) into the plan's input buffer
int tri_stage(bartels_tri_plan p, int model, const double *q, const double *dphi, const double *area,
              const double *params, double **dq, double **dd, double **da, double **dp) {
  bartels_ctx ctx = p->ctx;
  const size_t nV = p->nV, nT = p->nT;
  BT_CHECK(p->w_in.ensure(sizeof(double) * (2 * nV + 9 * nT + 8)));
  double *base = p->w_in.as<double>();
  *dq = base;
  *dd = base + 2 * nV;
  *da = *dd + 6 * nT;
  *dp = *da + nT;
  std::vector<double> pb;
  if (params) tri_params(model, params, p->nT, pb);
  if (q) BT_CUDA(cudaMemcpyAsync(*dq, q, sizeof(double) * 2 * nV, cudaMemcpyHostToDevice, ctx->stream));
  if (dphi) BT_CUDA(cudaMemcpyAsync(*dd, dphi, sizeof(double) * 6 * nT, cudaMemcpyHostToDevice, ctx->stream));
  BT_CUDA(cudaMemcpyAsync(*da, area, sizeof(double) * nT, cudaMemcpyHostToDevice, ctx->stream));
  if (params) BT_CUDA(cudaMemcpyAsync(*dp, pb.data(), sizeof(double) * 2 * nT, cudaMemcpyHostToDevice, ctx->stream));
  BT_CUDA(cudaStreamSynchronize(ctx->stream));  // pb is host memory on this stack frame
  return BARTELS_OK;
}

bool valid_tri_model(int m) { return m >= 0 && m <= 5; }
// energy and gradient: the reference has no tri2d linear-elasticity energy (its
// law is written for a displacement gradient, not the embedded F)
bool valid_tri_energy_model(int m) { return valid_tri_model(m) && m != BARTELS_LINEAR_ELASTICITY; }

}  // namespace
}  // namespace bartels

using namespace bartels;

extern "C" {

int bartels_tri_plan_create(bartels_ctx ctx, int nV, int nT, const int *E, int dim, bartels_tri_plan *out) {
  if (!ctx || !E || !out || nV <= 0 || nT <= 0 || (dim != 2 && dim != 3))
    return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  // incidences pack (tri << 2 | local index) into an int
  if ((int64_t)nT >= (1 << 29)) return fail(BARTELS_E_UNSUPPORTED, "too many triangles");
  BT_CUDA(cudaSetDevice(ctx->device));
  std::vector<int4> E4(nT);
  for (int t = 0; t < nT; ++t) {
    E4[t] = make_int4(E[t], E[t + (size_t)nT], E[t + 2 * (size_t)nT], 0);
    const int id[3] = {E4[t].x, E4[t].y, E4[t].z};
    for (int a = 0; a < 3; ++a)
      if (id[a] < 0 || id[a] >= nV) return fail(BARTELS_E_INVALID_ARG, "element index out of range");
  }
  // rows: sorted neighbours (self included); incidences in tri order
  std::vector<std::vector<int>> rows(nV);
  std::vector<int> inc_ptr(nV + 1, 0);
  for (int t = 0; t < nT; ++t) {
    const int id[3] = {E4[t].x, E4[t].y, E4[t].z};
    for (int a = 0; a < 3; ++a) {
      inc_ptr[id[a] + 1]++;
      for (int b = 0; b < 3; ++b) rows[id[a]].push_back(id[b]);
    }
  }
  for (int v = 0; v < nV; ++v) inc_ptr[v + 1] += inc_ptr[v];
  std::vector<int> inc(inc_ptr[nV]), fillp(inc_ptr.begin(), inc_ptr.end() - 1);
  for (int t = 0; t < nT; ++t) {
    const int id[3] = {E4[t].x, E4[t].y, E4[t].z};
    for (int a = 0; a < 3; ++a) inc[fillp[id[a]]++] = (t << 2) | a;
  }
  std::vector<int> brp(nV + 1, 0);
  for (int v = 0; v < nV; ++v) {
    std::vector<int> &r = rows[v];
    std::sort(r.begin(), r.end());
    r.erase(std::unique(r.begin(), r.end()), r.end());
    if (r.empty()) r.push_back(v);  // an unreferenced vertex keeps its diagonal block
    if (r.size() > 255) return fail(BARTELS_E_UNSUPPORTED, "a vertex has more than 254 neighbours");
    brp[v + 1] = brp[v] + (int)r.size();
  }
  std::vector<int> bcol(brp[nV]);
  std::vector<uint32_t> inc_pos(inc.size());
  for (int v = 0; v < nV; ++v) {
    std::copy(rows[v].begin(), rows[v].end(), bcol.begin() + brp[v]);
    for (int k = inc_ptr[v]; k < inc_ptr[v + 1]; ++k) {
      const int4 e = E4[inc[k] >> 2];
      const int id[3] = {e.x, e.y, e.z};
      uint32_t pos = 0;
      for (int b = 0; b < 3; ++b)
        pos |= (uint32_t)(std::lower_bound(rows[v].begin(), rows[v].end(), id[b]) - rows[v].begin()) << (8 * b);
      inc_pos[k] = pos;
    }
  }
  if ((int64_t)dim * dim * brp[nV] > (int64_t)INT32_MAX) return fail(BARTELS_E_UNSUPPORTED, "more than 2^31 CSR entries");
  auto p = new bartels_tri_plan_s();
  p->ctx = ctx;
  p->dim = dim;
  p->nV = nV;
  p->nT = nT;
  p->nnzb = brp[nV];
  p->h_brp = brp;
  p->h_bcol = bcol;
  int s = tri_upload(ctx, &p->E, E4.data(), E4.size());
  if (s == BARTELS_OK) s = tri_upload(ctx, &p->brp, brp.data(), brp.size());
  if (s == BARTELS_OK) s = tri_upload(ctx, &p->bcol, bcol.data(), bcol.size());
  if (s == BARTELS_OK) s = tri_upload(ctx, &p->inc_ptr, inc_ptr.data(), inc_ptr.size());
  if (s == BARTELS_OK) s = tri_upload(ctx, &p->inc, inc.data(), inc.size());
  if (s == BARTELS_OK) s = tri_upload(ctx, &p->inc_pos, inc_pos.data(), inc_pos.size());
  if (s == BARTELS_OK && cudaStreamSynchronize(ctx->stream) != cudaSuccess)
    s = fail(BARTELS_E_DEVICE, "tri2d plan upload failed");
  if (s != BARTELS_OK) {
    bartels_tri_plan_destroy(p);
    return s;
  }
  *out = p;
  return BARTELS_OK;
}

void bartels_tri_plan_destroy(bartels_tri_plan p) {
  if (!p) return;
  void *ptrs[] = {p->E, p->brp, p->bcol, p->inc_ptr, p->inc, p->inc_pos};
  for (void *q : ptrs)
    if (q) cudaFree(q);
  p->w_in.release();
  p->w_elem.release();
  p->w_out.release();
  delete p;
}

int bartels_tri_plan_csr_size(bartels_tri_plan p, int *n, int64_t *nnz) {
  if (!p) return fail(BARTELS_E_INVALID_ARG, "null plan");
  if (n) *n = p->dim * p->nV;
  if (nnz) *nnz = (int64_t)p->dim * p->dim * p->nnzb;
  return BARTELS_OK;
}

int bartels_tri_plan_csr_pattern(bartels_tri_plan p, int *row_ptr, int *col_idx) {
  if (!p) return fail(BARTELS_E_INVALID_ARG, "null plan");
  const int D = p->dim;
  for (int v = 0; v < p->nV; ++v) {
    const int rb = p->h_brp[v], nb = p->h_brp[v + 1] - rb;
    for (int kk = 0; kk < D; ++kk) {
      const int r = D * v + kk, start = D * D * rb + kk * D * nb;
      if (row_ptr) row_ptr[r] = start;
      if (col_idx)
        for (int j = 0; j < nb; ++j)
          for (int ll = 0; ll < D; ++ll) col_idx[start + D * j + ll] = D * p->h_bcol[rb + j] + ll;
    }
  }
  if (row_ptr) row_ptr[D * p->nV] = (int)((int64_t)D * D * p->nnzb);
  return BARTELS_OK;
}

int bartels_tri2dmesh_dphi_dX(bartels_ctx ctx, int nV, const double *V, int nT, const int *E, double *dphidX,
                              double *area) {
  if (!ctx || !V || !E || (!dphidX && !area) || nV <= 0 || nT <= 0) return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  BT_CUDA(cudaSetDevice(ctx->device));
  std::vector<int4> E4(nT);
  for (int t = 0; t < nT; ++t) {
    E4[t] = make_int4(E[t], E[t + (size_t)nT], E[t + 2 * (size_t)nT], 0);
    if (E4[t].x < 0 || E4[t].x >= nV || E4[t].y < 0 || E4[t].y >= nV || E4[t].z < 0 || E4[t].z >= nV)
      return fail(BARTELS_E_INVALID_ARG, "element index out of range");
  }
  // staging: V (2 nV), dphi (6 nT), area (nT) as doubles, then E at the next 16-byte boundary
  const size_t ndoubles = 2 * (size_t)nV + 7 * (size_t)nT;
  const size_t e_off = (sizeof(double) * ndoubles + 15) & ~size_t(15);
  BT_CHECK(ctx->stage_d.ensure(e_off + sizeof(int4) * nT));
  double *dV = ctx->stage_d.as<double>(), *dd = dV + 2 * (size_t)nV, *da = dd + 6 * (size_t)nT;
  int4 *dE = reinterpret_cast<int4 *>(reinterpret_cast<char *>(ctx->stage_d.p) + e_off);
  BT_CUDA(cudaMemcpyAsync(dV, V, sizeof(double) * 2 * nV, cudaMemcpyHostToDevice, ctx->stream));
  BT_CUDA(cudaMemcpyAsync(dE, E4.data(), sizeof(int4) * nT, cudaMemcpyHostToDevice, ctx->stream));
  BT_LAUNCH(ctx, k_tri2d_dphi, grid1(ctx, nT), 256, 0, nV, nT, dV, dE, dd, da);
  if (dphidX) BT_CUDA(cudaMemcpyAsync(dphidX, dd, sizeof(double) * 6 * nT, cudaMemcpyDeviceToHost, ctx->stream));
  if (area) BT_CUDA(cudaMemcpyAsync(area, da, sizeof(double) * nT, cudaMemcpyDeviceToHost, ctx->stream));
  BT_CUDA(cudaStreamSynchronize(ctx->stream));
  return BARTELS_OK;
}

int bartels_tri2dmesh_q(bartels_ctx ctx, bartels_tri_plan p, int model, const double *q, const double *dphidX,
                        const double *area, const double *params, double *energy) {
  BT_CHECK(check_tri(ctx, p, 2));
  if (!valid_tri_energy_model(model) || !q || !dphidX || !area || !params || !energy)
    return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  double *dq, *dd, *da, *dp;
  BT_CHECK(tri_stage(p, model, q, dphidX, area, params, &dq, &dd, &da, &dp));
  BT_CHECK(p->w_elem.ensure(sizeof(double) * (size_t)p->nT));
  BT_LAUNCH(ctx, k_tri2d_elem, grid1(ctx, p->nT), 256, 0, 0, model, p->nT, p->E, dq, dd, da, dp, 0, 0.0,
            p->w_elem.as<double>());
  std::vector<double> e(p->nT);
  BT_CUDA(cudaMemcpyAsync(e.data(), p->w_elem.p, sizeof(double) * p->nT, cudaMemcpyDeviceToHost, ctx->stream));
  BT_CUDA(cudaStreamSynchronize(ctx->stream));
  double s = 0.0;  // element order, as the scalar assemble (src/assemble.cpp:134-150)
  for (double x : e) s += x;
  *energy = s;
  if (!std::isfinite(s)) return fail(BARTELS_E_NONFINITE, "energy is not finite (J <= 0 for Neo-Hookean?)");
  return BARTELS_OK;
}

int bartels_tri2dmesh_dq(bartels_ctx ctx, bartels_tri_plan p, int model, const double *q, const double *dphidX,
                         const double *area, const double *params, double *g) {
  BT_CHECK(check_tri(ctx, p, 2));
  if (!valid_tri_energy_model(model) || !q || !dphidX || !area || !params || !g)
    return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  double *dq, *dd, *da, *dp;
  BT_CHECK(tri_stage(p, model, q, dphidX, area, params, &dq, &dd, &da, &dp));
  BT_CHECK(p->w_elem.ensure(sizeof(double) * 6 * (size_t)p->nT));
  BT_CHECK(p->w_out.ensure(sizeof(double) * 2 * (size_t)p->nV));
  BT_LAUNCH(ctx, k_tri2d_elem, grid1(ctx, p->nT), 256, 0, 1, model, p->nT, p->E, dq, dd, da, dp, 0, 0.0,
            p->w_elem.as<double>());
  BT_LAUNCH(ctx, k_tri2d_gather_vec, grid1(ctx, p->nV), 256, 0, p->nV, p->inc_ptr, p->inc, p->w_elem.as<double>(),
            p->w_out.as<double>());
  BT_CUDA(cudaMemcpyAsync(g, p->w_out.p, sizeof(double) * 2 * p->nV, cudaMemcpyDeviceToHost, ctx->stream));
  BT_CUDA(cudaStreamSynchronize(ctx->stream));
  for (int i = 0; i < 2 * p->nV; ++i)
    if (!std::isfinite(g[i])) return fail(BARTELS_E_NONFINITE, "gradient is not finite");
  return BARTELS_OK;
}

int bartels_tri2dmesh_dq2(bartels_ctx ctx, bartels_tri_plan p, int model, const double *q, const double *dphidX,
                          const double *area, const double *params, int psd_mode, double psd_tol,
                          double *csr_values) {
  BT_CHECK(check_tri(ctx, p, 2));
  if (!valid_tri_model(model) || !q || !dphidX || !area || !params || !csr_values ||
      (psd_mode != BARTELS_PSD_NONE && psd_mode != BARTELS_PSD_SIMPLE_FIX))
    return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  double *dq, *dd, *da, *dp;
  BT_CHECK(tri_stage(p, model, q, dphidX, area, params, &dq, &dd, &da, &dp));
  BT_CHECK(p->w_elem.ensure(sizeof(double) * 36 * (size_t)p->nT));
  BT_CHECK(p->w_out.ensure(sizeof(double) * 4 * (size_t)p->nnzb));
  BT_LAUNCH(ctx, k_tri2d_elem, grid1(ctx, p->nT), 256, 0, 2, model, p->nT, p->E, dq, dd, da, dp,
            psd_mode == BARTELS_PSD_SIMPLE_FIX ? 1 : 0, psd_tol, p->w_elem.as<double>());
  BT_LAUNCH(ctx, k_tri_gather_mat<2>, grid1(ctx, p->nV), 256, 0, p->nV, p->brp, p->inc_ptr, p->inc, p->inc_pos,
            p->w_elem.as<double>(), p->w_out.as<double>());
  BT_CUDA(cudaMemcpyAsync(csr_values, p->w_out.p, sizeof(double) * 4 * p->nnzb, cudaMemcpyDeviceToHost,
                          ctx->stream));
  BT_CUDA(cudaStreamSynchronize(ctx->stream));
  return BARTELS_OK;
}

int bartels_tri2dmesh_mass_matrix(bartels_ctx ctx, bartels_tri_plan p, const double *density, const double *area,
                                  double *csr_values) {
  BT_CHECK(check_tri(ctx, p, 2));
  if (!density || !area || !csr_values) return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  double *dq, *dd, *da, *dp;
  BT_CHECK(tri_stage(p, 0, nullptr, nullptr, area, nullptr, &dq, &dd, &da, &dp));
  // density goes where the params would be
  BT_CUDA(cudaMemcpyAsync(dp, density, sizeof(double) * p->nT, cudaMemcpyHostToDevice, ctx->stream));
  BT_CHECK(p->w_elem.ensure(sizeof(double) * 36 * (size_t)p->nT));
  BT_CHECK(p->w_out.ensure(sizeof(double) * 4 * (size_t)p->nnzb));
  BT_LAUNCH(ctx, k_tri2d_mass, grid1(ctx, p->nT), 256, 0, p->nT, dp, da, p->w_elem.as<double>());
  BT_LAUNCH(ctx, k_tri_gather_mat<2>, grid1(ctx, p->nV), 256, 0, p->nV, p->brp, p->inc_ptr, p->inc, p->inc_pos,
            p->w_elem.as<double>(), p->w_out.as<double>());
  BT_CUDA(cudaMemcpyAsync(csr_values, p->w_out.p, sizeof(double) * 4 * p->nnzb, cudaMemcpyDeviceToHost,
                          ctx->stream));
  BT_CUDA(cudaStreamSynchronize(ctx->stream));
  return BARTELS_OK;
}

int bartels_tri3dmesh_dphi_dX(bartels_ctx ctx, int nV, const double *V, int nT, const int *E, double *dphidX,
                              double *area) {
  if (!ctx || !V || !E || (!dphidX && !area) || nV <= 0 || nT <= 0) return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  BT_CUDA(cudaSetDevice(ctx->device));
  std::vector<int4> E4(nT);
  for (int t = 0; t < nT; ++t) {
    E4[t] = make_int4(E[t], E[t + (size_t)nT], E[t + 2 * (size_t)nT], 0);
    if (E4[t].x < 0 || E4[t].x >= nV || E4[t].y < 0 || E4[t].y >= nV || E4[t].z < 0 || E4[t].z >= nV)
      return fail(BARTELS_E_INVALID_ARG, "element index out of range");
  }
  // staging: V (3 nV), dphi (9 nT), area (nT) as doubles, then E at the next 16-byte boundary
  const size_t ndoubles = 3 * (size_t)nV + 10 * (size_t)nT;
  const size_t e_off = (sizeof(double) * ndoubles + 15) & ~size_t(15);
  BT_CHECK(ctx->stage_d.ensure(e_off + sizeof(int4) * nT));
  double *dV = ctx->stage_d.as<double>(), *dd = dV + 3 * (size_t)nV, *da = dd + 9 * (size_t)nT;
  int4 *dE = reinterpret_cast<int4 *>(reinterpret_cast<char *>(ctx->stage_d.p) + e_off);
  BT_CUDA(cudaMemcpyAsync(dV, V, sizeof(double) * 3 * nV, cudaMemcpyHostToDevice, ctx->stream));
  BT_CUDA(cudaMemcpyAsync(dE, E4.data(), sizeof(int4) * nT, cudaMemcpyHostToDevice, ctx->stream));
  BT_LAUNCH(ctx, k_tri3d_dphi, grid1(ctx, nT), 256, 0, nV, nT, dV, dE, dd, da);
  if (dphidX) BT_CUDA(cudaMemcpyAsync(dphidX, dd, sizeof(double) * 9 * nT, cudaMemcpyDeviceToHost, ctx->stream));
  if (area) BT_CUDA(cudaMemcpyAsync(area, da, sizeof(double) * nT, cudaMemcpyDeviceToHost, ctx->stream));
  BT_CUDA(cudaStreamSynchronize(ctx->stream));
  return BARTELS_OK;
}

int bartels_tri3dmesh_stvk_dq2(bartels_ctx ctx, bartels_tri_plan p, const double *q, const double *dphidX,
                               const double *N, const double *n, const double *dndq, const double *area,
                               const double *params, int psd_mode, double psd_tol, double *csr_values) {
  BT_CHECK(check_tri(ctx, p, 3));
  if (!q || !dphidX || !N || !n || !dndq || !area || !params || !csr_values ||
      (psd_mode != BARTELS_PSD_NONE && psd_mode != BARTELS_PSD_SIMPLE_FIX))
    return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  const size_t nV = p->nV, nT = p->nT;
  // inputs: q (3 nV), dphi (9 nT), N (3 nT), n (3 nT), dndq (27 nT), area (nT), params (2 nT)
  BT_CHECK(p->w_in.ensure(sizeof(double) * (3 * nV + 45 * nT + 8)));
  double *dq = p->w_in.as<double>(), *dd = dq + 3 * nV, *dN = dd + 9 * nT, *dn = dN + 3 * nT, *ddn = dn + 3 * nT,
         *da = ddn + 27 * nT, *dp = da + nT;
  BT_CUDA(cudaMemcpyAsync(dq, q, sizeof(double) * 3 * nV, cudaMemcpyHostToDevice, ctx->stream));
  BT_CUDA(cudaMemcpyAsync(dd, dphidX, sizeof(double) * 9 * nT, cudaMemcpyHostToDevice, ctx->stream));
  BT_CUDA(cudaMemcpyAsync(dN, N, sizeof(double) * 3 * nT, cudaMemcpyHostToDevice, ctx->stream));
  BT_CUDA(cudaMemcpyAsync(dn, n, sizeof(double) * 3 * nT, cudaMemcpyHostToDevice, ctx->stream));
  BT_CUDA(cudaMemcpyAsync(ddn, dndq, sizeof(double) * 27 * nT, cudaMemcpyHostToDevice, ctx->stream));
  BT_CUDA(cudaMemcpyAsync(da, area, sizeof(double) * nT, cudaMemcpyHostToDevice, ctx->stream));
  BT_CUDA(cudaMemcpyAsync(dp, params, sizeof(double) * 2 * nT, cudaMemcpyHostToDevice, ctx->stream));
  BT_CHECK(p->w_elem.ensure(sizeof(double) * 81 * nT));
  BT_CHECK(p->w_out.ensure(sizeof(double) * 9 * (size_t)p->nnzb));
  BT_LAUNCH(ctx, k_tri3d_stvk_hess, grid1(ctx, p->nT), 256, 0, p->nT, p->E, dq, dd, dN, dn, ddn, da, dp,
            psd_mode == BARTELS_PSD_SIMPLE_FIX ? 1 : 0, psd_tol, p->w_elem.as<double>());
  BT_LAUNCH(ctx, k_tri_gather_mat<3>, grid1(ctx, p->nV), 256, 0, p->nV, p->brp, p->inc_ptr, p->inc, p->inc_pos,
            p->w_elem.as<double>(), p->w_out.as<double>());
  BT_CUDA(cudaMemcpyAsync(csr_values, p->w_out.p, sizeof(double) * 9 * p->nnzb, cudaMemcpyDeviceToHost,
                          ctx->stream));
  BT_CUDA(cudaStreamSynchronize(ctx->stream));
  return BARTELS_OK;
}

#define BT_TRI_NAMED(name, M)                                                                                    \
  int bartels_tri2dmesh_##name##_q(bartels_ctx c, bartels_tri_plan p, const double *q, const double *d,       \
                                   const double *a, const double *pr, double *e) {                               \
    return bartels_tri2dmesh_q(c, p, M, q, d, a, pr, e);                                                        \
  }                                                                                                             \
  int bartels_tri2dmesh_##name##_dq(bartels_ctx c, bartels_tri_plan p, const double *q, const double *d,      \
                                    const double *a, const double *pr, double *g) {                              \
    return bartels_tri2dmesh_dq(c, p, M, q, d, a, pr, g);                                                       \
  }                                                                                                             \
  int bartels_tri2dmesh_##name##_dq2(bartels_ctx c, bartels_tri_plan p, const double *q, const double *d,     \
                                     const double *a, const double *pr, int psd, double tol, double *vals) {     \
    return bartels_tri2dmesh_dq2(c, p, M, q, d, a, pr, psd, tol, vals);                                         \
  }
BT_TRI_NAMED(neohookean, BARTELS_NEOHOOKEAN)
BT_TRI_NAMED(stvk, BARTELS_STVK)
BT_TRI_NAMED(corotational, BARTELS_COROTATIONAL)
BT_TRI_NAMED(arap, BARTELS_ARAP)
#undef BT_TRI_NAMED

int bartels_tri2dmesh_linear_elasticity_dq2(bartels_ctx c, bartels_tri_plan p, const double *q, const double *d,
                                            const double *a, const double *pr, int psd, double tol, double *vals) {
  return bartels_tri2dmesh_dq2(c, p, BARTELS_LINEAR_ELASTICITY, q, d, a, pr, psd, tol, vals);
}

}  // extern "C"
