// CPU baseline of the Newton path: the oracle's FP64 element math (the
// reference's formulas, bartels_oracle.hpp) driven the way the reference's
// Newton loop drives it (include/optimization_gradient_based.h:77-106,
// src/linesearch_backtracking_bisection.cpp:17-30), with OpenMP over elements
// and vertices and a precomputed CSR pattern + scatter positions instead of a
// triplet sort (the "optimised CPU" variant), and block-Jacobi PCG in FP64 in
// place of Eigen::SparseLU (a direct factorisation of 2.7M DOF is impractical).
// simple_psd_fix uses the tridiagonal-QL eigen-solver (psd_fix_ql), the method
// class of the reference's Eigen::SelfAdjointEigenSolver. ob_faithful_dq2 is the
// reference's own structure on one thread (triplets, sort / compress).
//
// Test infrastructure and CPU timing only: timed by bench.py on the host cores and
// never used by the GPU library.
#include <omp.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "bartels_oracle.hpp"

using namespace oracle;

namespace {

struct Baseline {
  int nV = 0, nT = 0, model = 0;
  std::vector<int> E;           // nT x 4 row-major
  std::vector<double> X;        // 3 nV
  std::vector<double> dphi;     // nT x 12 (reference flatten)
  std::vector<double> vol;      // nT
  std::vector<double> params;   // nT x 2 row-major
  std::vector<double> density;  // nT
  // incidence lists and CSR pattern (scalar CSR of the 3x3 block pattern)
  std::vector<int> inc_ptr, inc_tet;
  std::vector<int> brp, bcol;
  std::vector<int64_t> rp;      // scalar row_ptr (3 nV + 1)
  std::vector<int> col;
  std::vector<int> pos;         // 16 block positions per tet: pos[16 t + 4 a + b]
  // problem
  std::vector<double> q_base, x_hat, f_ext;
  std::vector<unsigned char> pinned;
  double mass_coeff = 0, scale = 1, force_scale = 0, psd_tol = -1;
  // state
  std::vector<double> vals;     // CSR values
};

inline int64_t entry_index(const Baseline &B, int v, int j, int k, int l) {
  const int nb = B.brp[v + 1] - B.brp[v];
  return 9ll * B.brp[v] + 3ll * k * nb + 3ll * j + l;
}

void element_qe(const Baseline &B, const double *x, int t, double *qe) {
  for (int a = 0; a < 4; ++a) {
    const int v = B.E[4 * t + a];
    for (int d = 0; d < 3; ++d) qe[3 * a + d] = B.q_base[3 * v + d] + B.scale * x[3 * v + d];
  }
}

double now() { return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count(); }

}  // namespace

extern "C" {

void *ob_create(int nV, const double *V, int nT, const int *E) {
  auto B = new Baseline;
  B->nV = nV;
  B->nT = nT;
  B->E.resize(4 * (size_t)nT);
  for (int t = 0; t < nT; ++t)
    for (int a = 0; a < 4; ++a) B->E[4 * (size_t)t + a] = E[t + (size_t)nT * a];
  B->X.resize(3 * (size_t)nV);
  for (int v = 0; v < nV; ++v)
    for (int d = 0; d < 3; ++d) B->X[3 * (size_t)v + d] = V[v + (size_t)nV * d];
  B->dphi.resize(12 * (size_t)nT);
  B->vol.resize(nT);
#pragma omp parallel for schedule(static)
  for (int t = 0; t < nT; ++t) {
    const double *x[4];
    for (int a = 0; a < 4; ++a) x[a] = &B->X[3 * (size_t)B->E[4 * (size_t)t + a]];
    tet_dphi_dX(&B->dphi[12 * (size_t)t], x[0], x[1], x[2], x[3]);
    B->vol[t] = tet_volume(x[0], x[1], x[2], x[3]);
  }
  // incidences (tet order per vertex)
  B->inc_ptr.assign(nV + 1, 0);
  for (int t = 0; t < nT; ++t)
    for (int a = 0; a < 4; ++a) B->inc_ptr[B->E[4 * (size_t)t + a] + 1]++;
  for (int v = 0; v < nV; ++v) B->inc_ptr[v + 1] += B->inc_ptr[v];
  B->inc_tet.resize(4 * (size_t)nT);
  {
    std::vector<int> fill(B->inc_ptr.begin(), B->inc_ptr.end() - 1);
    for (int t = 0; t < nT; ++t)
      for (int a = 0; a < 4; ++a) B->inc_tet[fill[B->E[4 * (size_t)t + a]]++] = 4 * t + a;
  }
  // block pattern
  std::vector<std::vector<int>> rows(nV);
#pragma omp parallel for schedule(dynamic, 1024)
  for (int v = 0; v < nV; ++v) {
    auto &r = rows[v];
    r.push_back(v);
    for (int k = B->inc_ptr[v]; k < B->inc_ptr[v + 1]; ++k) {
      const int t = B->inc_tet[k] >> 2;
      for (int b = 0; b < 4; ++b) r.push_back(B->E[4 * (size_t)t + b]);
    }
    std::sort(r.begin(), r.end());
    r.erase(std::unique(r.begin(), r.end()), r.end());
  }
  B->brp.assign(nV + 1, 0);
  for (int v = 0; v < nV; ++v) B->brp[v + 1] = B->brp[v] + (int)rows[v].size();
  B->bcol.resize(B->brp[nV]);
  B->rp.resize(3 * (size_t)nV + 1);
  B->col.resize(9 * (size_t)B->brp[nV]);
#pragma omp parallel for schedule(static)
  for (int v = 0; v < nV; ++v) {
    const auto &r = rows[v];
    const int nb = (int)r.size();
    std::copy(r.begin(), r.end(), B->bcol.begin() + B->brp[v]);
    for (int k = 0; k < 3; ++k) {
      B->rp[3 * (size_t)v + k] = 9ll * B->brp[v] + 3ll * k * nb;
      for (int j = 0; j < nb; ++j)
        for (int l = 0; l < 3; ++l) B->col[9ll * B->brp[v] + 3ll * k * nb + 3 * j + l] = 3 * r[j] + l;
    }
  }
  B->rp[3 * (size_t)nV] = 9ll * B->brp[nV];
  B->pos.resize(16 * (size_t)nT);
#pragma omp parallel for schedule(static)
  for (int t = 0; t < nT; ++t)
    for (int a = 0; a < 4; ++a) {
      const int v = B->E[4 * (size_t)t + a];
      const auto &r = rows[v];
      for (int b = 0; b < 4; ++b)
        B->pos[16 * (size_t)t + 4 * a + b] =
            (int)(std::lower_bound(r.begin(), r.end(), B->E[4 * (size_t)t + b]) - r.begin());
    }
  B->params.assign(2 * (size_t)nT, 0.0);
  B->density.assign(nT, 0.0);
  B->q_base.assign(3 * (size_t)nV, 0.0);
  B->x_hat.assign(3 * (size_t)nV, 0.0);
  B->f_ext.assign(3 * (size_t)nV, 0.0);
  B->pinned.assign(nV, 0);
  B->vals.assign(B->col.size(), 0.0);
  return B;
}

void ob_free(void *h) { delete static_cast<Baseline *>(h); }
long long ob_nnz(void *h) { return (long long)static_cast<Baseline *>(h)->col.size(); }

// params: nT x 2 column-major (reference layout)
void ob_set(void *h, int model, const double *params, const double *density, const double *q_base,
            const double *x_hat, const double *f_ext, const unsigned char *pinned, double mass_coeff, double scale,
            double force_scale, double psd_tol) {
  auto B = static_cast<Baseline *>(h);
  B->model = model;
  for (int t = 0; t < B->nT; ++t) {
    B->params[2 * (size_t)t] = params[t];
    B->params[2 * (size_t)t + 1] = params[t + (size_t)B->nT];
  }
  if (density) std::copy(density, density + B->nT, B->density.begin());
  const size_t n = 3 * (size_t)B->nV;
  if (q_base) std::copy(q_base, q_base + n, B->q_base.begin());
  if (x_hat) std::copy(x_hat, x_hat + n, B->x_hat.begin());
  if (f_ext) std::copy(f_ext, f_ext + n, B->f_ext.begin());
  if (pinned) std::copy(pinned, pinned + B->nV, B->pinned.begin());
  B->mass_coeff = mass_coeff;
  B->scale = scale;
  B->force_scale = force_scale;
  B->psd_tol = psd_tol;
}

double ob_energy(void *h, const double *x) {
  auto B = static_cast<Baseline *>(h);
  double e = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : e)
  for (int t = 0; t < B->nT; ++t) {
    double qe[12];
    element_qe(*B, x, t, qe);
    e += element_q(B->model, qe, &B->dphi[12 * (size_t)t], &B->params[2 * (size_t)t], B->vol[t]);
    if (B->mass_coeff != 0.0) {
      const double m = B->density[t] * B->vol[t];
      for (int a = 0; a < 4; ++a)
        for (int b = 0; b < 4; ++b) {
          const double c = (a == b ? 0.1 : 0.05) * m;
          const int va = B->E[4 * (size_t)t + a], vb = B->E[4 * (size_t)t + b];
          for (int d = 0; d < 3; ++d)
            e += B->mass_coeff * c * x[3 * va + d] * (0.5 * x[3 * vb + d] - B->x_hat[3 * vb + d]);
        }
    }
  }
  double f = 0.0;
  const int n = 3 * B->nV;
#pragma omp parallel for schedule(static) reduction(+ : f)
  for (int i = 0; i < n; ++i) f += B->f_ext[i] * x[i];
  return e - B->force_scale * f;
}

void ob_gradient(void *h, const double *x, double *g) {
  auto B = static_cast<Baseline *>(h);
  std::vector<double> ge(12 * (size_t)B->nT);
#pragma omp parallel for schedule(static)
  for (int t = 0; t < B->nT; ++t) {
    double qe[12], out[12];
    element_qe(*B, x, t, qe);
    element_dq(B->model, out, qe, &B->dphi[12 * (size_t)t], &B->params[2 * (size_t)t], B->vol[t]);
    for (int i = 0; i < 12; ++i) out[i] *= B->scale;
    if (B->mass_coeff != 0.0) {
      const double m = B->density[t] * B->vol[t];
      for (int a = 0; a < 4; ++a)
        for (int b = 0; b < 4; ++b) {
          const double c = B->mass_coeff * (a == b ? 0.1 : 0.05) * m;
          const int vb = B->E[4 * (size_t)t + b];
          for (int d = 0; d < 3; ++d) out[3 * a + d] += c * (x[3 * vb + d] - B->x_hat[3 * vb + d]);
        }
    }
    std::memcpy(&ge[12 * (size_t)t], out, sizeof(out));
  }
#pragma omp parallel for schedule(static)
  for (int v = 0; v < B->nV; ++v) {
    double s[3] = {0, 0, 0};
    for (int k = B->inc_ptr[v]; k < B->inc_ptr[v + 1]; ++k) {
      const int ta = B->inc_tet[k];
      for (int d = 0; d < 3; ++d) s[d] += ge[12 * (size_t)(ta >> 2) + 3 * (ta & 3) + d];
    }
    for (int d = 0; d < 3; ++d) g[3 * v + d] = B->pinned[v] ? 0.0 : s[d] - B->force_scale * B->f_ext[3 * v + d];
  }
}

// Hessian contributions of tets [t0, t1) added into the CSR values (zeroed
// when clear != 0): mass_coeff M + scale^2 K (PSD-projected when psd_tol >= 0).
void ob_hessian(void *h, const double *x, int t0, int t1, int clear) {
  auto B = static_cast<Baseline *>(h);
  if (clear) std::fill(B->vals.begin(), B->vals.end(), 0.0);
  ElementFlags fl;
  const double s2 = B->scale * B->scale;
#pragma omp parallel for schedule(dynamic, 256)
  for (int t = t0; t < t1; ++t) {
    double qe[12], K[144];
    element_qe(*B, x, t, qe);
    element_dq2(B->model, K, qe, &B->dphi[12 * (size_t)t], &B->params[2 * (size_t)t], B->vol[t], fl);
    if (B->psd_tol >= 0) psd_fix_ql(K, 12, B->psd_tol);
    const double m = B->density[t] * B->vol[t];
    for (int a = 0; a < 4; ++a) {
      const int v = B->E[4 * (size_t)t + a];
      for (int b = 0; b < 4; ++b) {
        const int j = B->pos[16 * (size_t)t + 4 * a + b];
        for (int k = 0; k < 3; ++k)
          for (int l = 0; l < 3; ++l) {
            double val = s2 * K[(3 * a + k) + 12 * (3 * b + l)];
            if (k == l) val += B->mass_coeff * (a == b ? 0.1 : 0.05) * m;
#pragma omp atomic
            B->vals[entry_index(*B, v, j, k, l)] += val;
          }
      }
    }
  }
}

static void spmv(const Baseline &B, const double *x, double *y) {
  const int n = 3 * B.nV;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; ++i) {
    double s = 0.0;
    for (int64_t k = B.rp[i]; k < B.rp[i + 1]; ++k) s += B.vals[k] * x[B.col[k]];
    y[i] = B.pinned[i / 3] ? 0.0 : s;
  }
}

// Block-Jacobi PCG in FP64 on the current values: solve H x = b to
// ||r|| <= rel_tol ||b|| or max_it iterations. Returns iterations.
int ob_pcg(void *h, const double *b, double *x, double rel_tol, int max_it, double *rel_out) {
  auto B = static_cast<Baseline *>(h);
  const int nV = B->nV, n = 3 * nV;
  std::vector<double> minv(9 * (size_t)nV), r(n), z(n), p(n), ap(n);
#pragma omp parallel for schedule(static)
  for (int v = 0; v < nV; ++v) {
    const int nb = B->brp[v + 1] - B->brp[v];
    int jd = 0;
    while (B->bcol[B->brp[v] + jd] != v) ++jd;
    double A[9], G[9];
    for (int k = 0; k < 3; ++k)
      for (int l = 0; l < 3; ++l) A[k + 3 * l] = B->vals[9ll * B->brp[v] + 3ll * k * nb + 3 * jd + l];
    cofactor3(G, A);
    const double det = det3(A);
    for (int k = 0; k < 3; ++k)
      for (int l = 0; l < 3; ++l)
        minv[9 * (size_t)v + 3 * k + l] = (B->pinned[v] || det == 0.0) ? 0.0 : G[l + 3 * k] / det;
  }
  auto prec = [&](const std::vector<double> &in, std::vector<double> &out) {
#pragma omp parallel for schedule(static)
    for (int v = 0; v < nV; ++v)
      for (int k = 0; k < 3; ++k) {
        const double *m = &minv[9 * (size_t)v + 3 * k];
        out[3 * v + k] = m[0] * in[3 * v] + m[1] * in[3 * v + 1] + m[2] * in[3 * v + 2];
      }
  };
  auto dotv = [&](const std::vector<double> &a, const std::vector<double> &c) {
    double s = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : s)
    for (int i = 0; i < n; ++i) s += a[i] * c[i];
    return s;
  };
  spmv(*B, x, ap.data());
  double bb = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : bb)
  for (int i = 0; i < n; ++i) {
    r[i] = B->pinned[i / 3] ? 0.0 : b[i] - ap[i];
    bb += b[i] * b[i];
  }
  prec(r, z);
  p = z;
  double rz = dotv(r, z), rr = dotv(r, r);
  const double tol2 = rel_tol * rel_tol * bb;
  int it = 0;
  while (rr > tol2 && it < max_it) {
    spmv(*B, p.data(), ap.data());
    const double alpha = rz / dotv(p, ap);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
      x[i] += alpha * p[i];
      r[i] -= alpha * ap[i];
    }
    prec(r, z);
    const double rz_new = dotv(r, z);
    rr = dotv(r, r);
    const double beta = rz_new / rz;
    rz = rz_new;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
    ++it;
  }
  if (rel_out) *rel_out = bb > 0 ? std::sqrt(rr / bb) : 0.0;
  return it;
}

// One Newton iteration (gradient test skipped by the caller): Hessian on the
// tets [0, nT) (or a sample), PCG, the reference's line search. stats:
// [0] |g|, [1] pcg iterations, [2] line-search backtracks, [3] t_grad,
// [4] t_hess, [5] t_pcg, [6] t_ls, [7] alpha
void ob_newton_iteration(void *h, double *x, double pcg_rel_tol, int pcg_max_it, int ls_max, double *stats) {
  auto B = static_cast<Baseline *>(h);
  const int n = 3 * B->nV;
  std::vector<double> g(n), d(n, 0.0), b(n), xt(n);
  double t0 = now();
  ob_gradient(h, x, g.data());
  double gg = 0.0;
  for (int i = 0; i < n; ++i) gg += g[i] * g[i];
  double t1 = now();
  ob_hessian(h, x, 0, B->nT, 1);
  double t2 = now();
  for (int i = 0; i < n; ++i) b[i] = -g[i];
  int its = ob_pcg(h, b.data(), d.data(), pcg_rel_tol, pcg_max_it, nullptr);
  double t3 = now();
  double gd = 0.0;
  for (int i = 0; i < n; ++i) gd += g[i] * d[i];
  const double fx = ob_energy(h, x);
  double alpha = 1.0;
  int it = 0;
  for (;;) {
    for (int i = 0; i < n; ++i) xt[i] = x[i] + alpha * d[i];
    if (!(ob_energy(h, xt.data()) > fx + 1e-8 * gd && it < ls_max)) break;
    alpha *= 0.5;
    ++it;
  }
  for (int i = 0; i < n; ++i) x[i] += alpha * d[i];
  double t4 = now();
  if (stats) {
    stats[0] = std::sqrt(gg);
    stats[1] = its;
    stats[2] = it;
    stats[3] = t1 - t0;
    stats[4] = t2 - t1;
    stats[5] = t3 - t2;
    stats[6] = t4 - t3;
    stats[7] = alpha;
  }
}

// linear_tetmesh_{model}_dq2 with the simple_psd_fix callback in the
// reference's structure (src/linear_tetmesh_neohookean_dq2.cpp:17-27,
// src/assemble.cpp:57-94): per tet the dense 12x12, the projection, 144
// triplets; then setFromTriplets' sort / compress. Serial. Returns nnz and the
// sum and absolute sum of the values (for checking).
long long ob_faithful_dq2(int model, double psd_tol, int nV, int nT, const int *E, const double *q,
                          const double *dphidX, const double *vol, const double *params, double *sums) {
  CSR H;
  ElementFlags fl;
  assemble_matrix(H, nV, nT, E, [&](int t, double *K) {
    double qe[12], dphi[12], p[2];
    gather_qe(qe, q, E, nT, t);
    row_of(dphi, dphidX, nT, 12, t);
    row_of(p, params, nT, 2, t);
    element_dq2(model, K, qe, dphi, p, vol[t], fl);
    if (psd_tol >= 0) psd_fix_ql(K, 12, psd_tol);
  });
  double s = 0, a = 0;
  for (double v : H.val) {
    s += v;
    a += std::fabs(v);
  }
  if (sums) {
    sums[0] = s;
    sums[1] = a;
  }
  return (long long)H.val.size();
}

int ob_threads() { return omp_get_max_threads(); }
// Thread count of the parallel regions that follow on the calling thread
// (the reference-faithful variant times the PCG on one thread).
void ob_set_threads(int n) { omp_set_num_threads(n > 0 ? n : omp_get_num_procs()); }
double ob_wtime() { return now(); }

}  // extern "C"
