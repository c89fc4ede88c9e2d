// Drives the CPU oracle (oracle/oracle_capi.cpp) and the CPU baseline
// (oracle/oracle_baseline.cpp) through every entry point on a small jittered
// Kuhn cube, built with -fsanitize=address,undefined by the test suite: any
// out-of-bounds access, use after free, leak or undefined arithmetic aborts
// the run. Light self-checks keep the calls meaningful. Prints
// "oracle sanitize ok" and returns 0 on success.
#include <cmath>
#include <cstdio>
#include <vector>

extern "C" {
void or_dphi_dX(int nV, const double *V, int nT, const int *E, double *dphidX);
void or_volume(int nV, const double *V, int nT, const int *E, double *vol);
double or_tetmesh_q(int model, int nT, const int *E, const double *q, const double *dphidX, const double *vol,
                    const double *params);
void or_tetmesh_dq(int model, int nV, int nT, const int *E, const double *q, const double *dphidX,
                   const double *vol, const double *params, double *g);
void *or_tetmesh_dq2(int model, int psd_mode, double psd_tol, int corot_layout, int nV, int nT, const int *E,
                     const double *q, const double *dphidX, const double *vol, const double *params);
void *or_mass_matrix(int nV, int nT, const int *E, const double *density, const double *vol);
void *or_fixed_point_constraint(int nV, int dim, const int *fixed, int nfix);
int or_find_min_vertices(int nV, const double *V, int dim, double tol, int *out);
int or_csr_rows(void *h);
long long or_csr_nnz(void *h);
void or_csr_copy(void *h, int *row_ptr, int *col, double *val);
void or_csr_free(void *h);
int or_psd_fix_ql(double *A, int n, double tol);
void or_psd_fix(double *A, int n, double tol);
void *ob_create(int nV, const double *V, int nT, const int *E);
void ob_free(void *h);
void ob_set(void *h, int model, const double *params, const double *density, const double *q_base,
            const double *x_hat, const double *f_ext, const unsigned char *pinned, double mass_coeff, double scale,
            double force_scale, double psd_tol);
double ob_energy(void *h, const double *x);
void ob_gradient(void *h, const double *x, double *g);
void ob_hessian(void *h, const double *x, int t0, int t1, int clear);
int ob_pcg(void *h, const double *b, double *x, double rel_tol, int max_it, double *rel_out);
void ob_newton_iteration(void *h, double *x, double pcg_rel_tol, int pcg_max_it, int ls_max, double *stats);
long long ob_faithful_dq2(int model, double psd_tol, int nV, int nT, const int *E, const double *q,
                          const double *dphidX, const double *vol, const double *params, double *sums);
}

#define REQUIRE(c)                                                          \
  do {                                                                      \
    if (!(c)) {                                                             \
      std::fprintf(stderr, "check failed: %s (line %d)\n", #c, __LINE__); \
      return 1;                                                             \
    }                                                                       \
  } while (0)

int main() {
  const int n = 3, m = n + 1, nV = m * m * m, nT = 6 * n * n * n;
  std::vector<double> V(3 * (size_t)nV);  // column-major nV x 3
  unsigned seed = 7;
  auto rnd = [&] {
    seed = seed * 1103515245u + 12345u;
    return ((seed >> 8) & 0xFFFF) / 65536.0 - 0.5;
  };
  for (int k = 0; k < m; ++k)
    for (int j = 0; j < m; ++j)
      for (int i = 0; i < m; ++i) {
        const int v = i + m * (j + m * k);
        V[v] = i / (double)n + 0.02 * rnd() / n;
        V[v + nV] = j / (double)n + 0.02 * rnd() / n;
        V[v + 2 * nV] = k / (double)n;
      }
  const int perms[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
  const int sgn[6] = {1, -1, -1, 1, 1, -1};
  const int step[3] = {1, m, m * m};
  std::vector<int> E(4 * (size_t)nT);  // column-major nT x 4
  int t = 0;
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i)
        for (int p = 0; p < 6; ++p, ++t) {
          const int p0 = i + m * (j + m * k), p1 = p0 + step[perms[p][0]], p2 = p1 + step[perms[p][1]],
                    p3 = p2 + step[perms[p][2]];
          E[t] = p0;
          E[t + nT] = sgn[p] > 0 ? p1 : p2;
          E[t + 2 * nT] = sgn[p] > 0 ? p2 : p1;
          E[t + 3 * nT] = p3;
        }
  std::vector<double> dphi(12 * (size_t)nT), vol(nT), params(2 * (size_t)nT), rho(nT, 1000.0), q(3 * (size_t)nV);
  or_dphi_dX(nV, V.data(), nT, E.data(), dphi.data());
  or_volume(nV, V.data(), nT, E.data(), vol.data());
  for (int e = 0; e < nT; ++e) {
    REQUIRE(vol[e] > 0);
    params[e] = 3e5;
    params[e + nT] = 1e6;
  }
  for (int v = 0; v < nV; ++v)
    for (int d = 0; d < 3; ++d) q[3 * v + d] = V[v + (size_t)nV * d] * (d == 2 ? 0.8 : 1.05) + 0.01 * rnd() / n;
  std::vector<double> g(3 * (size_t)nV);
  for (int model = 0; model <= 5; ++model) {
    const double e = or_tetmesh_q(model, nT, E.data(), q.data(), dphi.data(), vol.data(), params.data());
    REQUIRE(std::isfinite(e));
    or_tetmesh_dq(model, nV, nT, E.data(), q.data(), dphi.data(), vol.data(), params.data(), g.data());
    for (int psd = 0; psd < 2; ++psd) {
      void *h = or_tetmesh_dq2(model, psd, 1e-6, 1, nV, nT, E.data(), q.data(), dphi.data(), vol.data(),
                               params.data());
      const int rows = or_csr_rows(h);
      const long long nnz = or_csr_nnz(h);
      std::vector<int> rp(rows + 1), col(nnz);
      std::vector<double> val(nnz);
      or_csr_copy(h, rp.data(), col.data(), val.data());
      or_csr_free(h);
      REQUIRE(rows == 3 * nV && rp[rows] == nnz);
      double sums[2];
      REQUIRE(ob_faithful_dq2(model, psd ? 1e-6 : -1.0, nV, nT, E.data(), q.data(), dphi.data(), vol.data(),
                              params.data(), sums) == nnz);
    }
  }
  void *M = or_mass_matrix(nV, nT, E.data(), rho.data(), vol.data());
  REQUIRE(or_csr_rows(M) == 3 * nV);
  or_csr_free(M);
  std::vector<int> bottom(nV);
  const int nb = or_find_min_vertices(nV, V.data(), 2, 1e-3, bottom.data());
  REQUIRE(nb == m * m);
  void *P = or_fixed_point_constraint(nV, 3, bottom.data(), nb);
  REQUIRE(or_csr_rows(P) == 3 * (nV - nb));
  or_csr_free(P);
  // the two simple_psd_fix solvers on an indefinite 12 x 12
  double A[144], B[144];
  for (int i = 0; i < 12; ++i)
    for (int j = 0; j <= i; ++j) A[i + 12 * j] = A[j + 12 * i] = rnd() + (i == j ? 0.1 * (i - 6) : 0.0);
  for (int i = 0; i < 144; ++i) B[i] = A[i];
  REQUIRE(or_psd_fix_ql(A, 12, 1e-6) == 1);
  or_psd_fix(B, 12, 1e-6);
  for (int i = 0; i < 144; ++i) REQUIRE(std::fabs(A[i] - B[i]) < 1e-10);
  // CPU baseline: one implicit-Euler Newton iteration, PSD-projected
  std::vector<unsigned char> pinned(nV, 0);
  for (int i = 0; i < nb; ++i) pinned[bottom[i]] = 1;
  std::vector<double> xhat(3 * (size_t)nV, 0.0), fext(3 * (size_t)nV, 0.0), x(3 * (size_t)nV, 0.0);
  for (int v = 0; v < nV; ++v) fext[3 * v + 2] = -9.81;
  for (int v = 0; v < nV; ++v)
    for (int d = 0; d < 3; ++d) q[3 * v + d] = V[v + (size_t)nV * d];
  void *cb = ob_create(nV, V.data(), nT, E.data());
  ob_set(cb, 0, params.data(), rho.data(), q.data(), xhat.data(), fext.data(), pinned.data(), 1.0, 0.01, 0.01, 1e-6);
  REQUIRE(std::isfinite(ob_energy(cb, x.data())));
  ob_gradient(cb, x.data(), g.data());
  ob_hessian(cb, x.data(), 0, nT, 1);
  std::vector<double> d(3 * (size_t)nV, 0.0), b(3 * (size_t)nV);
  for (size_t i = 0; i < b.size(); ++i) b[i] = -g[i];
  double rel = 0.0;
  REQUIRE(ob_pcg(cb, b.data(), d.data(), 1e-8, 2000, &rel) > 0 && rel <= 1e-8);
  double stats[8];
  ob_newton_iteration(cb, x.data(), 1e-8, 2000, 50, stats);
  REQUIRE(std::isfinite(stats[0]));
  ob_free(cb);
  std::printf("oracle sanitize ok\n");
  return 0;
}
