// Triangle meshes in the plane (linear_tri2dmesh_* of the reference): per-element
// energy, gradient and Hessian of every material law, mass matrix, and the
// deterministic assembly into a CSR whose pattern (2x2 vertex blocks, rows 2v
// and 2v+1 with the sorted columns of v's neighbours) is the reference's.
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

struct bartels_tri2d_plan_s {
  bartels_ctx ctx = nullptr;
  int nV = 0, nT = 0;
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

template <class Fn>
__device__ __forceinline__ void tri_law(int model, const double *F, const double *pv, Fn &&fn) {
  switch (model) {
    case MODEL_NH: fn(LawNH<double>(F, pv)); break;
    case MODEL_NH_ISO: fn(LawNHIso<double>(F, pv)); break;
    case MODEL_STVK: fn(LawStVK<double>(F, pv)); break;
    case MODEL_LE: fn(LawLE<double>(F, pv)); break;
    case MODEL_ARAP: {
      double pa[2];
      arap_pv(pv, pa);
      fn(LawCorot<double>(F, pa, false));
      break;
    }
    default: fn(LawCorot<double>(F, pv, false)); break;
  }
}

// Symmetric 6x6 (row-major, in place) -> W max(L, tol) W^T: cyclic Jacobi until
// the off-diagonal mass is at rounding level (at most 40 sweeps).
__device__ void psd_fix6(double *A, double tol) {
  double W[36];
  for (int i = 0; i < 36; ++i) W[i] = (i % 7 == 0) ? 1.0 : 0.0;
  for (int s = 0; s < 40; ++s) {
    double off = 0.0, dia = 0.0;
    for (int i = 0; i < 6; ++i) {
      dia += A[7 * i] * A[7 * i];
      for (int j = 0; j < i; ++j) off += A[6 * i + j] * A[6 * i + j];
    }
    if (off <= 1e-32 * dia) break;
    for (int p = 0; p < 5; ++p)
      for (int r = p + 1; r < 6; ++r) {
        const double apr = A[6 * p + r];
        if (apr == 0.0) continue;
        const double theta = (A[6 * r + r] - A[6 * p + p]) / (2.0 * apr);
        const double t = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        const double c = 1.0 / sqrt(t * t + 1.0), sn = t * c;
        for (int k = 0; k < 6; ++k) {  // columns p, r
          const double akp = A[6 * k + p], akr = A[6 * k + r];
          A[6 * k + p] = c * akp - sn * akr;
          A[6 * k + r] = sn * akp + c * akr;
        }
        for (int k = 0; k < 6; ++k) {  // rows p, r
          const double apk = A[6 * p + k], ark = A[6 * r + k];
          A[6 * p + k] = c * apk - sn * ark;
          A[6 * r + k] = sn * apk + c * ark;
        }
        for (int k = 0; k < 6; ++k) {
          const double wkp = W[6 * k + p], wkr = W[6 * k + r];
          W[6 * k + p] = c * wkp - sn * wkr;
          W[6 * k + r] = sn * wkp + c * wkr;
        }
      }
  }
  double L[6];
  for (int i = 0; i < 6; ++i) L[i] = A[7 * i] < tol ? tol : A[7 * i];
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) {
      double s = 0.0;
      for (int k = 0; k < 6; ++k) s += W[6 * i + k] * L[k] * W[6 * j + k];
      A[6 * i + j] = s;
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
      tri_law(model, el.F, el.pv, [&](const auto &law) {
        for (int a = 0; a < 3; ++a)
          for (int b = 0; b < 3; ++b) {
            double B3[9];
            law.block(el.phi[a], el.phi[b], B3);
            for (int k = 0; k < 2; ++k)
              for (int l = 0; l < 2; ++l) K[6 * (2 * a + k) + 2 * b + l] = B3[3 * k + l];
          }
      });
      if (psd) psd_fix6(K, tol);
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

// Row pair (2v, 2v + 1) of the CSR: every entry summed over the vertex's tris in
// tri order (as setFromTriplets sums duplicates, src/assemble.cpp:57-94). The
// thread owns its rows' segment [4 brp[v], 4 brp[v + 1]) of the values.
__global__ void k_tri2d_gather_mat(int nV, const int *__restrict__ brp, const int *__restrict__ inc_ptr,
                                   const int *__restrict__ inc, const uint32_t *__restrict__ inc_pos,
                                   const double *__restrict__ ke, double *__restrict__ vals) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nV; v += gridDim.x * blockDim.x) {
    const int rb = brp[v], rs = 2 * (brp[v + 1] - rb);
    double *row = vals + 4ll * rb;
    for (int i = 0; i < 2 * rs; ++i) row[i] = 0.0;
    for (int k = inc_ptr[v]; k < inc_ptr[v + 1]; ++k) {
      const int ta = inc[k], t = ta >> 2, a = ta & 3;
      const uint32_t pos = inc_pos[k];
      const double *K = ke + 36ll * t;
      for (int b = 0; b < 3; ++b) {
        const int j = (pos >> (8 * b)) & 255;
        for (int kk = 0; kk < 2; ++kk)
          for (int ll = 0; ll < 2; ++ll) row[kk * rs + 2 * j + ll] += K[6 * (2 * a + kk) + 2 * b + ll];
      }
    }
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

int check_tri(bartels_ctx ctx, bartels_tri2d_plan p) {
  if (!ctx || !p) return fail(BARTELS_E_INVALID_ARG, "null context or plan");
  if (p->ctx != ctx) return fail(BARTELS_E_INVALID_ARG, "plan belongs to another context");
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
int tri_stage(bartels_tri2d_plan p, int model, const double *q, const double *dphi, const double *area,
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

int bartels_tri2d_plan_create(bartels_ctx ctx, int nV, int nT, const int *E, bartels_tri2d_plan *out) {
  if (!ctx || !E || !out || nV <= 0 || nT <= 0) return fail(BARTELS_E_INVALID_ARG, "bad arguments");
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
  if ((int64_t)nT >= (1 << 29)) return fail(BARTELS_E_UNSUPPORTED, "too many triangles");
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
  if (4 * (int64_t)brp[nV] > (int64_t)INT32_MAX) return fail(BARTELS_E_UNSUPPORTED, "more than 2^31 CSR entries");
  auto p = new bartels_tri2d_plan_s();
  p->ctx = ctx;
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
    bartels_tri2d_plan_destroy(p);
    return s;
  }
  *out = p;
  return BARTELS_OK;
}

void bartels_tri2d_plan_destroy(bartels_tri2d_plan p) {
  if (!p) return;
  void *ptrs[] = {p->E, p->brp, p->bcol, p->inc_ptr, p->inc, p->inc_pos};
  for (void *q : ptrs)
    if (q) cudaFree(q);
  p->w_in.release();
  p->w_elem.release();
  p->w_out.release();
  delete p;
}

int bartels_tri2d_plan_csr_size(bartels_tri2d_plan p, int *n, int64_t *nnz) {
  if (!p) return fail(BARTELS_E_INVALID_ARG, "null plan");
  if (n) *n = 2 * p->nV;
  if (nnz) *nnz = 4 * p->nnzb;
  return BARTELS_OK;
}

int bartels_tri2d_plan_csr_pattern(bartels_tri2d_plan p, int *row_ptr, int *col_idx) {
  if (!p) return fail(BARTELS_E_INVALID_ARG, "null plan");
  for (int v = 0; v < p->nV; ++v) {
    const int rb = p->h_brp[v], nb = p->h_brp[v + 1] - rb;
    for (int kk = 0; kk < 2; ++kk) {
      const int r = 2 * v + kk, start = 4 * rb + kk * 2 * nb;
      if (row_ptr) row_ptr[r] = start;
      if (col_idx)
        for (int j = 0; j < nb; ++j) {
          col_idx[start + 2 * j] = 2 * p->h_bcol[rb + j];
          col_idx[start + 2 * j + 1] = 2 * p->h_bcol[rb + j] + 1;
        }
    }
  }
  if (row_ptr) row_ptr[2 * p->nV] = (int)(4 * p->nnzb);
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

int bartels_tri2dmesh_q(bartels_ctx ctx, bartels_tri2d_plan p, int model, const double *q, const double *dphidX,
                        const double *area, const double *params, double *energy) {
  BT_CHECK(check_tri(ctx, p));
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

int bartels_tri2dmesh_dq(bartels_ctx ctx, bartels_tri2d_plan p, int model, const double *q, const double *dphidX,
                         const double *area, const double *params, double *g) {
  BT_CHECK(check_tri(ctx, p));
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

int bartels_tri2dmesh_dq2(bartels_ctx ctx, bartels_tri2d_plan p, int model, const double *q, const double *dphidX,
                          const double *area, const double *params, int psd_mode, double psd_tol,
                          double *csr_values) {
  BT_CHECK(check_tri(ctx, p));
  if (!valid_tri_model(model) || !q || !dphidX || !area || !params || !csr_values ||
      (psd_mode != BARTELS_PSD_NONE && psd_mode != BARTELS_PSD_SIMPLE_FIX))
    return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  double *dq, *dd, *da, *dp;
  BT_CHECK(tri_stage(p, model, q, dphidX, area, params, &dq, &dd, &da, &dp));
  BT_CHECK(p->w_elem.ensure(sizeof(double) * 36 * (size_t)p->nT));
  BT_CHECK(p->w_out.ensure(sizeof(double) * 4 * (size_t)p->nnzb));
  BT_LAUNCH(ctx, k_tri2d_elem, grid1(ctx, p->nT), 256, 0, 2, model, p->nT, p->E, dq, dd, da, dp,
            psd_mode == BARTELS_PSD_SIMPLE_FIX ? 1 : 0, psd_tol, p->w_elem.as<double>());
  BT_LAUNCH(ctx, k_tri2d_gather_mat, grid1(ctx, p->nV), 256, 0, p->nV, p->brp, p->inc_ptr, p->inc, p->inc_pos,
            p->w_elem.as<double>(), p->w_out.as<double>());
  BT_CUDA(cudaMemcpyAsync(csr_values, p->w_out.p, sizeof(double) * 4 * p->nnzb, cudaMemcpyDeviceToHost,
                          ctx->stream));
  BT_CUDA(cudaStreamSynchronize(ctx->stream));
  return BARTELS_OK;
}

int bartels_tri2dmesh_mass_matrix(bartels_ctx ctx, bartels_tri2d_plan p, const double *density, const double *area,
                                  double *csr_values) {
  BT_CHECK(check_tri(ctx, p));
  if (!density || !area || !csr_values) return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  double *dq, *dd, *da, *dp;
  BT_CHECK(tri_stage(p, 0, nullptr, nullptr, area, nullptr, &dq, &dd, &da, &dp));
  // density goes where the params would be
  BT_CUDA(cudaMemcpyAsync(dp, density, sizeof(double) * p->nT, cudaMemcpyHostToDevice, ctx->stream));
  BT_CHECK(p->w_elem.ensure(sizeof(double) * 36 * (size_t)p->nT));
  BT_CHECK(p->w_out.ensure(sizeof(double) * 4 * (size_t)p->nnzb));
  BT_LAUNCH(ctx, k_tri2d_mass, grid1(ctx, p->nT), 256, 0, p->nT, dp, da, p->w_elem.as<double>());
  BT_LAUNCH(ctx, k_tri2d_gather_mat, grid1(ctx, p->nV), 256, 0, p->nV, p->brp, p->inc_ptr, p->inc, p->inc_pos,
            p->w_elem.as<double>(), p->w_out.as<double>());
  BT_CUDA(cudaMemcpyAsync(csr_values, p->w_out.p, sizeof(double) * 4 * p->nnzb, cudaMemcpyDeviceToHost,
                          ctx->stream));
  BT_CUDA(cudaStreamSynchronize(ctx->stream));
  return BARTELS_OK;
}

#define BT_TRI_NAMED(name, M)                                                                                    \
  int bartels_tri2dmesh_##name##_q(bartels_ctx c, bartels_tri2d_plan p, const double *q, const double *d,       \
                                   const double *a, const double *pr, double *e) {                               \
    return bartels_tri2dmesh_q(c, p, M, q, d, a, pr, e);                                                        \
  }                                                                                                             \
  int bartels_tri2dmesh_##name##_dq(bartels_ctx c, bartels_tri2d_plan p, const double *q, const double *d,      \
                                    const double *a, const double *pr, double *g) {                              \
    return bartels_tri2dmesh_dq(c, p, M, q, d, a, pr, g);                                                       \
  }                                                                                                             \
  int bartels_tri2dmesh_##name##_dq2(bartels_ctx c, bartels_tri2d_plan p, const double *q, const double *d,     \
                                     const double *a, const double *pr, int psd, double tol, double *vals) {     \
    return bartels_tri2dmesh_dq2(c, p, M, q, d, a, pr, psd, tol, vals);                                         \
  }
BT_TRI_NAMED(neohookean, BARTELS_NEOHOOKEAN)
BT_TRI_NAMED(stvk, BARTELS_STVK)
BT_TRI_NAMED(corotational, BARTELS_COROTATIONAL)
BT_TRI_NAMED(arap, BARTELS_ARAP)
#undef BT_TRI_NAMED

int bartels_tri2dmesh_linear_elasticity_dq2(bartels_ctx c, bartels_tri2d_plan p, const double *q, const double *d,
                                            const double *a, const double *pr, int psd, double tol, double *vals) {
  return bartels_tri2dmesh_dq2(c, p, BARTELS_LINEAR_ELASTICITY, q, d, a, pr, psd, tol, vals);
}

}  // extern "C"
