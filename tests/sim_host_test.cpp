// Host-only parts of the sim:: layer (include/bartels_sim.hpp) linked against
// the library, run without a GPU: row-ordered values moved into compressed
// columns (checked with unsymmetric values), the fixed-point constraint
// matrix in compressed columns, find_min_vertices appending like the
// reference, and the host line search. Prints "sim host ok", returns 0.
#include <cmath>
#include <cstdio>
#include <vector>

#include "bartels_sim.hpp"

#define REQUIRE(c)                                                          \
  do {                                                                      \
    if (!(c)) {                                                             \
      std::fprintf(stderr, "check failed: %s (line %d)\n", #c, __LINE__); \
      return 1;                                                             \
    }                                                                       \
  } while (0)

int main() {
  // 4 x 4 symmetric pattern (tridiagonal plus (0, 3)); row-ordered values
  // v(i, j) = 10 i + j, deliberately unsymmetric
  sim::SparseMatrix S;
  S.n_rows = S.n_cols = 4;
  const int rows[4][3] = {{0, 1, 3}, {0, 1, 2}, {1, 2, 3}, {0, 2, 3}};
  S.outer_ptr = {0};
  for (int r = 0; r < 4; ++r) {
    for (int c : rows[r]) {
      S.inner_idx.push_back(c);
      S.values.push_back(10.0 * r + c);
    }
    S.outer_ptr.push_back((int)S.inner_idx.size());
  }
  sim::detail::row_values_to_columns(S);
  for (int c = 0; c < 4; ++c)  // column c, row inner_idx[k]: H(row, c) = 10 row + c
    for (int k = S.outer_ptr[c]; k < S.outer_ptr[c + 1]; ++k) REQUIRE(S.values[k] == 10.0 * S.inner_idx[k] + c);
  // and back to rows (what the solver's C ABI takes): row r holds H(r, c) = 10 r + c
  std::vector<int> rp, ci;
  std::vector<double> rv;
  sim::detail::columns_to_rows(S, rp, ci, rv);
  REQUIRE(rp == S.outer_ptr && ci == S.inner_idx);
  for (int rr = 0; rr < 4; ++rr)
    for (int k = rp[rr]; k < rp[rr + 1]; ++k) REQUIRE(rv[k] == 10.0 * rr + ci[k]);
  // constraint matrix: 4 vertices in 3D, vertices 1 and 3 fixed -> 6 x 12, compressed columns
  sim::MatrixXd V(4, 3);
  for (int v = 0; v < 4; ++v)
    for (int d = 0; d < 3; ++d) V(v, d) = (d == 2) ? (v % 2 ? 0.0 : 1.0) : v;
  sim::MatrixXi fixed(2, 1);
  fixed(0) = 1;
  fixed(1) = 3;
  sim::SparseMatrix P;
  sim::fixed_point_constraint_matrix(P, V, fixed);
  REQUIRE(P.rows() == 6 && P.cols() == 12 && P.nonZeros() == 6 && (int)P.outer_ptr.size() == 13);
  int r = 0;
  for (int c = 0; c < 12; ++c) {
    const bool free_dof = (c / 3 != 1 && c / 3 != 3);
    REQUIRE(P.outer_ptr[c + 1] - P.outer_ptr[c] == (free_dof ? 1 : 0));
    if (free_dof) {
      REQUIRE(P.inner_idx[P.outer_ptr[c]] == r && P.values[P.outer_ptr[c]] == 1.0);
      ++r;
    }
  }
  // find_min_vertices appends the vertices on the minimum of coordinate 2
  std::vector<int> idx = {42};
  sim::find_min_vertices(idx, V, 2);
  REQUIRE(idx.size() == 3 && idx[0] == 42 && idx[1] == 1 && idx[2] == 3);
  // line search on a quadratic, host objective
  auto quad = [](const sim::VectorXd &x) {
    double s = 0;
    for (int i = 0; i < x.rows(); ++i) s += 0.5 * x.data()[i] * x.data()[i];
    return s;
  };
  sim::VectorXd x(3, 1), g(3, 1), d(3, 1);
  for (int i = 0; i < 3; ++i) {
    x(i) = 1.0 + i;
    g(i) = x(i);
    d(i) = -x(i);
  }
  REQUIRE(sim::linesearch_backtracking_bisection(x, d, quad, g, 100, 1.0, 1e-4, 0.5) == sim::CONVERGED);
  REQUIRE(std::fabs(x(2)) < 1e-15);
  std::printf("sim host ok\n");
  return 0;
}
