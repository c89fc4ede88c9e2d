// C entry points of the FP64 CPU oracle (test infrastructure only; see the
// header of bartels_oracle.hpp). Loaded by tests through ctypes.
#include "bartels_oracle.hpp"

#include <cstdlib>
#include <memory>

using namespace oracle;

namespace {
struct Handle {
  CSR m;
};
}  // namespace

extern "C" {

// linear_tetmesh_dphi_dX, src/linear_tetmesh_dphi_dX.cpp:5-18 via
// src/eval_at_point.cpp:49-54: one row of 12 per tet.
void or_dphi_dX(int nV, const double *V, int nT, const int *E, double *dphidX) {
  for (int t = 0; t < nT; ++t) {
    double X[4][3], out[12];
    for (int a = 0; a < 4; ++a) {
      int v = E[t + (size_t)nT * a];
      for (int d = 0; d < 3; ++d) X[a][d] = V[v + (size_t)nV * d];
    }
    tet_dphi_dX(out, X[0], X[1], X[2], X[3]);
    for (int c = 0; c < 12; ++c) dphidX[t + (size_t)nT * c] = out[c];
  }
}

void or_volume(int nV, const double *V, int nT, const int *E, double *vol) {
  for (int t = 0; t < nT; ++t) {
    double X[4][3];
    for (int a = 0; a < 4; ++a) {
      int v = E[t + (size_t)nT * a];
      for (int d = 0; d < 3; ++d) X[a][d] = V[v + (size_t)nV * d];
    }
    vol[t] = tet_volume(X[0], X[1], X[2], X[3]);
  }
}

// linear_tetmesh_{model}_q: scalar assemble, serial left-to-right sum from
// element 0 (src/assemble.cpp:134-150).
double or_tetmesh_q(int model, int nT, const int *E, const double *q, const double *dphidX,
                    const double *vol, const double *params) {
  double energy = 0;
  for (int t = 0; t < nT; ++t) {
    double qe[12], dphi[12], p[2];
    gather_qe(qe, q, E, nT, t);
    row_of(dphi, dphidX, nT, 12, t);
    row_of(p, params, nT, 2, t);
    double e = element_q(model, qe, dphi, p, vol[t]);
    energy = (t == 0) ? e : energy + e;
  }
  return energy;
}

// per-element energies (for per-element parity checks)
void or_tetmesh_q_elements(int model, int nT, const int *E, const double *q, const double *dphidX,
                           const double *vol, const double *params, double *out) {
  for (int t = 0; t < nT; ++t) {
    double qe[12], dphi[12], p[2];
    gather_qe(qe, q, E, nT, t);
    row_of(dphi, dphidX, nT, 12, t);
    row_of(p, params, nT, 2, t);
    out[t] = element_q(model, qe, dphi, p, vol[t]);
  }
}

// linear_tetmesh_{model}_dq: vector assemble, serial scatter-add in element
// order (src/assemble.cpp:113-129).
void or_tetmesh_dq(int model, int nV, int nT, const int *E, const double *q, const double *dphidX,
                   const double *vol, const double *params, double *g) {
  for (int i = 0; i < 3 * nV; ++i) g[i] = 0.0;
  for (int t = 0; t < nT; ++t) {
    double qe[12], dphi[12], p[2], ge[12];
    gather_qe(qe, q, E, nT, t);
    row_of(dphi, dphidX, nT, 12, t);
    row_of(p, params, nT, 2, t);
    element_dq(model, ge, qe, dphi, p, vol[t]);
    for (int a = 0; a < 4; ++a)
      for (int d = 0; d < 3; ++d) g[3 * E[t + (size_t)nT * a] + d] += ge[3 * a + d];
  }
}

// linear_tetmesh_{model}_dq2 with an optional simple_psd_fix element callback
// (src/linear_tetmesh_neohookean_dq2.cpp:17-27, src/simple_psd_fix.cpp).
// psd_mode: 0 none, 1 simple_psd_fix(tol). corot_layout: 1 reference, 0 exact.
void *or_tetmesh_dq2(int model, int psd_mode, double psd_tol, int corot_layout, int nV, int nT, const int *E,
                     const double *q, const double *dphidX, const double *vol, const double *params) {
  auto h = new Handle;
  ElementFlags fl;
  fl.corot_layout_reference = corot_layout != 0;
  assemble_matrix(h->m, nV, nT, E, [&](int t, double *K) {
    double qe[12], dphi[12], p[2];
    gather_qe(qe, q, E, nT, t);
    row_of(dphi, dphidX, nT, 12, t);
    row_of(p, params, nT, 2, t);
    element_dq2(model, K, qe, dphi, p, vol[t], fl);
    if (psd_mode == 1) psd_fix(K, 12, psd_tol);
  });
  return h;
}

// per-element 12x12 blocks (col-major, 144 per tet) for element-level parity
void or_tetmesh_dq2_elements(int model, int psd_mode, double psd_tol, int corot_layout, int nT, const int *E,
                             const double *q, const double *dphidX, const double *vol, const double *params,
                             double *out) {
  ElementFlags fl;
  fl.corot_layout_reference = corot_layout != 0;
  for (int t = 0; t < nT; ++t) {
    double qe[12], dphi[12], p[2];
    gather_qe(qe, q, E, nT, t);
    row_of(dphi, dphidX, nT, 12, t);
    row_of(p, params, nT, 2, t);
    element_dq2(model, out + (size_t)144 * t, qe, dphi, p, vol[t], fl);
    if (psd_mode == 1) psd_fix(out + (size_t)144 * t, 12, psd_tol);
  }
}

// linear_tetmesh_mass_matrix, src/linear_tetmesh_mass_matrix.cpp:14-22 with
// linear_tet_mass_matrix, src/linear_tet_mass_matrix.cpp:12-42:
// m = rho vol; diagonal blocks m/10 I, off-diagonal blocks m/20 I.
void *or_mass_matrix(int nV, int nT, const int *E, const double *density, const double *vol) {
  auto h = new Handle;
  assemble_matrix(h->m, nV, nT, E, [&](int t, double *K) {
    double mass = density[t] * vol[t];
    double c0 = (1.0 / 10.0) * mass, c1 = (1.0 / 20.0) * mass;
    for (int i = 0; i < 12; ++i)
      for (int j = 0; j < 12; ++j) K[i + 12 * j] = (i % 3 == j % 3) ? ((i / 3 == j / 3) ? c0 : c1) : 0.0;
  });
  return h;
}

// linear_tetmesh_const_ext_force, src/linear_tetmesh_const_ext_force.cpp:9-16
// with linear_tet_const_ext_force, src/linear_tet_const_ext_force.cpp:8-9.
void or_const_ext_force(int nV, int nT, const int *E, const double *vol, const double *traction, double *f) {
  for (int i = 0; i < 3 * nV; ++i) f[i] = 0.0;
  for (int t = 0; t < nT; ++t)
    for (int a = 0; a < 4; ++a)
      for (int d = 0; d < 3; ++d) f[3 * E[t + (size_t)nT * a] + d] += traction[d] * (0.25 * vol[t]);
}

// fixed_point_constraint_matrix, src/fixed_point_constraint_matrix.cpp:12-36.
// fixed must be sorted ascending (the reference's single-pass merge needs it).
void *or_fixed_point_constraint(int nV, int dim, const int *fixed, int nfix) {
  std::vector<Triplet> trip;
  int q_size = nV * dim, stride = dim;
  int jj = 0;
  for (int ii = 0; ii < q_size; ii += stride) {
    if (jj < nfix && fixed[jj] == ii / stride) {
      jj += 1;
    } else {
      for (int kk = 0; kk < stride; ++kk) trip.push_back({ii - stride * jj + kk, ii + kk, 1.0});
    }
  }
  auto h = new Handle;
  triplets_to_csr(h->m, q_size - stride * nfix, trip);
  return h;
}

// find_min_vertices, src/find_min_vertices.cpp:8-19 (V column-major nV x 3).
int or_find_min_vertices(int nV, const double *V, int dim, double tol, int *out) {
  double mn = V[0 + (size_t)nV * dim];
  for (int v = 0; v < nV; ++v) mn = std::min(mn, V[v + (size_t)nV * dim]);
  int k = 0;
  for (int v = 0; v < nV; ++v)
    if (std::fabs(V[v + (size_t)nV * dim] - mn) <= tol) out[k++] = v;
  return k;
}

// CSR handle access
int or_csr_rows(void *h) { return static_cast<Handle *>(h)->m.n; }
long long or_csr_nnz(void *h) { return (long long)static_cast<Handle *>(h)->m.col.size(); }
void or_csr_copy(void *h, int *row_ptr, int *col, double *val) {
  auto &m = static_cast<Handle *>(h)->m;
  std::copy(m.row_ptr.begin(), m.row_ptr.end(), row_ptr);
  std::copy(m.col.begin(), m.col.end(), col);
  std::copy(m.val.begin(), m.val.end(), val);
}
void or_csr_free(void *h) { delete static_cast<Handle *>(h); }

// element-level math
double or_psi(int model, const double *F, const double *p) { return model_psi(model, F, p); }
void or_dpsi(int model, const double *F, const double *p, double *P) { model_dpsi(model, P, F, p); }
void or_d2psi(int model, const double *F, const double *p, int corot_layout, double *H) {
  ElementFlags fl;
  fl.corot_layout_reference = corot_layout != 0;
  model_d2psi(model, H, F, p, fl);
}
void or_d2psi_corot_dsvd_literal(const double *F, const double *p, double *H) {
  d2psi_corot_dsvd_literal(H, F, p);
}
void or_svd3(const double *F, double *U, double *S, double *V) { svd3(F, U, S, V); }
void or_psd_fix(double *A, int n, double tol) { psd_fix(A, n, tol); }
int or_psd_fix_ql(double *A, int n, double tol) { return psd_fix_ql(A, n, tol) ? 1 : 0; }
void or_build_B(const double *dphi12, double *B) { build_B(B, dphi12); }

}  // extern "C"
