// C++ caller of the sim:: layer (include/bartels_sim.hpp) written the way a
// user of the reference's headers would: builds a 2x2x2 Kuhn cube, evaluates
// q / dq / dq2 (with simple_psd_fix), mass, force, the constraint matrix, a
// search direction, a line search and the pointwise laws, and checks them
// against each other.
// Prints "sim shim ok" and returns 0 on success.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "bartels_sim.hpp"

#define REQUIRE(c)                                                   \
  do {                                                               \
    if (!(c)) {                                                      \
      std::fprintf(stderr, "check failed: %s (line %d)\n", #c, __LINE__); \
      return 1;                                                      \
    }                                                                \
  } while (0)

static sim::VectorXd params2_stvk(double lam, double mu) {
  sim::VectorXd p(2, 1);
  p(0) = lam;
  p(1) = mu;
  return p;
}

int main() {
  const int n = 2, m = n + 1;
  sim::MatrixXd V(m * m * m, 3);
  for (int k = 0; k < m; ++k)
    for (int j = 0; j < m; ++j)
      for (int i = 0; i < m; ++i) {
        const int v = i + m * (j + m * k);
        V(v, 0) = i * 0.5;
        V(v, 1) = j * 0.5;
        V(v, 2) = k * 0.5;
      }
  // 6 Kuhn tets per cell along the (0,0,0)-(1,1,1) diagonal, positively oriented
  const int perms[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
  const int sgn[6] = {1, -1, -1, 1, 1, -1};
  const int step[3] = {1, m, m * m};
  sim::MatrixXi E(6 * n * n * n, 4);
  int t = 0;
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i)
        for (int p = 0; p < 6; ++p) {
          const int p0 = i + m * (j + m * k), p1 = p0 + step[perms[p][0]], p2 = p1 + step[perms[p][1]],
                    p3 = p2 + step[perms[p][2]];
          E(t, 0) = p0;
          E(t, 1) = sgn[p] > 0 ? p1 : p2;
          E(t, 2) = sgn[p] > 0 ? p2 : p1;
          E(t, 3) = p3;
          ++t;
        }
  const int nV = V.rows(), nT = E.rows();
  sim::MatrixXd dphidX;
  sim::linear_tetmesh_dphi_dX(dphidX, V, E);
  REQUIRE(dphidX.rows() == nT && dphidX.cols() == 12);
  sim::VectorXd vol(nT, 1), density(nT, 1);
  for (int e = 0; e < nT; ++e) {
    vol(e) = 0.125 / 6.0;
    density(e) = 1000.0;
  }
  const double Y = 2e6, nu = 0.45, lam = Y * nu / ((1 + nu) * (1 - 2 * nu)), mu = Y / (2 * (1 + nu));
  sim::MatrixXd params(nT, 2);
  for (int e = 0; e < nT; ++e) {
    params(e, 0) = 0.5 * mu;
    params(e, 1) = 0.5 * lam;
  }
  sim::VectorXd q(3 * nV, 1);
  for (int v = 0; v < nV; ++v)
    for (int d = 0; d < 3; ++d) q(3 * v + d) = V(v, d) * (d == 2 ? 0.97 : 1.01) + 0.003 * std::sin(7.0 * v + d);

  const double e0 = sim::linear_tetmesh_neohookean_q(V, E, q, dphidX, vol, params);
  sim::VectorXd g;
  sim::linear_tetmesh_neohookean_dq(g, V, E, q, dphidX, vol, params);
  REQUIRE(std::isfinite(e0) && e0 > 0);
  // gradient against centred differences of the energy (src/finite_differences.cpp:42-80)
  for (int i = 0; i < 3 * nV; i += 7) {
    const double h = 1e-6;
    sim::VectorXd qp = q, qm = q;
    qp(i) += h;
    qm(i) -= h;
    const double fd = (sim::linear_tetmesh_neohookean_q(V, E, qp, dphidX, vol, params) -
                       sim::linear_tetmesh_neohookean_q(V, E, qm, dphidX, vol, params)) /
                      (2 * h);
    REQUIRE(std::fabs(fd - g(i)) <= 1e-4 * (std::fabs(g(i)) + 1.0));
  }
  sim::SparseMatrix H;
  sim::linear_tetmesh_neohookean_dq2(H, V, E, q, dphidX, vol, params, sim::simple_psd_fix(1e-6));
  REQUIRE(H.rows() == 3 * nV && H.nonZeros() == H.outer_ptr.back());
  // ARAP through the same names (k in params column 0)
  sim::SparseMatrix Ha;
  sim::linear_tetmesh_arap_dq2(Ha, V, E, q, dphidX, vol, params, sim::simple_psd_fix(1e-6));
  REQUIRE(Ha.nonZeros() == H.nonZeros());
  REQUIRE(sim::linear_tetmesh_arap_q(V, E, q, dphidX, vol, params) >= 0.0);
  sim::SparseMatrix M;
  sim::linear_tetmesh_mass_matrix(M, V, E, density, vol);
  double msum = 0;
  for (double v : M.values) msum += v;
  REQUIRE(std::fabs(msum - 3 * 1000.0) < 1e-9);  // 3 x total mass
  sim::VectorXd f;
  sim::VectorXd traction(3, 1);
  traction(2) = -9810.0;
  sim::linear_tetmesh_const_ext_force(f, V, E, vol, traction);
  double fz = 0;
  for (int v = 0; v < nV; ++v) fz += f(3 * v + 2);
  REQUIRE(std::fabs(fz + 9810.0) < 1e-8);
  sim::MatrixXi fixed(m * m, 1);
  for (int i = 0; i < m * m; ++i) fixed(i) = i;  // the z = 0 face
  sim::SparseMatrix P;
  sim::fixed_point_constraint_matrix(P, V, fixed);
  REQUIRE(P.rows() == 3 * (nV - m * m) && P.cols() == 3 * nV);
  // search direction on H + M (SPD), residual check
  sim::SparseMatrix A = H;
  for (size_t k = 0; k < A.values.size(); ++k) A.values[k] += M.values[k];
  sim::PCGSolver solver;
  sim::VectorXd d;
  REQUIRE(sim::search_direction_newton_sparse(d, g, A, solver));
  // A d + g with A in compressed columns (column c, rows inner_idx)
  std::vector<double> Ad(A.rows(), 0.0);
  for (int c = 0; c < A.cols(); ++c)
    for (int k = A.outer_ptr[c]; k < A.outer_ptr[c + 1]; ++k) Ad[A.inner_idx[k]] += A.values[k] * d(c);
  double rr = 0, gg = 0;
  for (int i = 0; i < A.rows(); ++i) {
    rr += (Ad[i] + g(i)) * (Ad[i] + g(i));
    gg += g(i) * g(i);
  }
  REQUIRE(std::sqrt(rr) <= 2e-8 * std::sqrt(gg));
  // line search along -g on a quadratic
  auto quad = [&](const sim::VectorXd &x) {
    double s = 0;
    for (int i = 0; i < x.rows(); ++i) s += 0.5 * x.data()[i] * x.data()[i];
    return s;
  };
  sim::VectorXd x(4, 1), gx(4, 1), dx(4, 1);
  for (int i = 0; i < 4; ++i) {
    x(i) = 1.0 + i;
    gx(i) = x(i);
    dx(i) = -3.0 * x(i);
  }
  REQUIRE(sim::linesearch_backtracking_bisection(x, dx, quad, gx, 100, 1.0, 1e-4, 0.5) == sim::CONVERGED);
  REQUIRE(std::fabs(x(0) - (1.0 - 1.5)) < 1e-12);
  // the same V / E buffers rewritten in place with the vertices relabelled
  // v -> nV - 1 - v: a new mesh at the old addresses, the same physical state
  {
    const sim::MatrixXd V0 = V;
    const sim::VectorXd q0 = q;
    for (int v = 0; v < nV; ++v)
      for (int d = 0; d < 3; ++d) {
        V(nV - 1 - v, d) = V0(v, d);
        q(3 * (nV - 1 - v) + d) = q0(3 * v + d);
      }
    for (int e = 0; e < nT; ++e)
      for (int a = 0; a < 4; ++a) E(e, a) = nV - 1 - E(e, a);
    const double e1 = sim::linear_tetmesh_neohookean_q(V, E, q, dphidX, vol, params);
    REQUIRE(std::fabs(e1 - e0) <= 1e-10 * e0);
    sim::VectorXd g1;
    sim::linear_tetmesh_neohookean_dq(g1, V, E, q, dphidX, vol, params);
    for (int v = 0; v < nV; ++v)
      for (int d = 0; d < 3; ++d)
        REQUIRE(std::fabs(g1(3 * (nV - 1 - v) + d) - g(3 * v + d)) <= 1e-9 * (std::fabs(g(3 * v + d)) + 1.0));
  }
  // pointwise laws (include/dpsi_neohookean_dF.h, include/d2psi_stvk_dF2.h):
  // dpsi against central differences of psi, d2psi against those of dpsi
  {
    sim::MatrixXd F(3, 3);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) F(i, j) = (i == j ? 1.0 : 0.0) + 0.05 * std::sin(3.0 * i + 5.0 * j + 1.0);
    sim::VectorXd p2(2, 1);
    p2(0) = 0.5 * mu;
    p2(1) = 0.5 * lam;
    sim::VectorXd dw;
    sim::dpsi_neohookean_dF(dw, F, p2);
    sim::MatrixXd ddw;
    sim::d2psi_stvk_dF2(ddw, F, params2_stvk(lam, mu));
    REQUIRE(dw.rows() == 9 && ddw.rows() == 9 && ddw.cols() == 9);
    const double h = 1e-6;
    for (int r = 0; r < 9; ++r) {
      sim::MatrixXd Fp = F, Fm = F;
      Fp.data()[r] += h;
      Fm.data()[r] -= h;
      const double fd = (sim::psi_neohookean_F(Fp, p2) - sim::psi_neohookean_F(Fm, p2)) / (2 * h);
      REQUIRE(std::fabs(fd - dw(r)) <= 1e-6 * mu);
      sim::VectorXd gp, gm;
      sim::dpsi_stvk_dF(gp, Fp, params2_stvk(lam, mu));
      sim::dpsi_stvk_dF(gm, Fm, params2_stvk(lam, mu));
      for (int c = 0; c < 9; ++c) REQUIRE(std::fabs((gp(c) - gm(c)) / (2 * h) - ddw(c, r)) <= 1e-6 * (lam + mu));
    }
  }
  // the reference's 2D case (tests/test_constitutive_model.cpp:107-135): one triangle at rest
  {
    sim::MatrixXd V2(3, 2);
    V2(0, 0) = 96.921; V2(0, 1) = 44.047;
    V2(1, 0) = 81.5;   V2(1, 1) = 37.5;
    V2(2, 0) = 87.452; V2(2, 1) = 31.207;
    sim::MatrixXi E2(1, 3);
    E2(0, 0) = 0; E2(0, 1) = 1; E2(0, 2) = 2;
    sim::MatrixXd params2(1, 2);
    params2(0, 0) = 6.2069e+06;
    params2(0, 1) = 6.8966e+05;
    sim::VectorXd area(1, 1);
    area(0) = 68.002;
    sim::VectorXd q2(6, 1);
    for (int v = 0; v < 3; ++v) {
      q2(2 * v) = V2(v, 0);
      q2(2 * v + 1) = V2(v, 1);
    }
    sim::MatrixXd dX2;
    sim::linear_tri2dmesh_dphi_dX(dX2, V2, E2);
    sim::VectorXd f2;
    sim::linear_tri2dmesh_corotational_dq(f2, V2, E2, q2, dX2, area, params2);
    for (int i = 0; i < 6; ++i) REQUIRE(std::fabs(f2(i)) <= 1e-6 * 6.2069e+06);
    sim::SparseMatrix H2;
    sim::linear_tri2dmesh_neohookean_dq2(H2, V2, E2, q2, dX2, area, params2, sim::simple_psd_fix(1e-6));
    REQUIRE(H2.rows() == 6 && H2.nonZeros() == 36);
  }
  std::printf("sim shim ok: energy %.6e, nnz %lld, pcg iterations %d\n", e0, (long long)H.nonZeros(),
              solver.report.iterations);
  return 0;
}
