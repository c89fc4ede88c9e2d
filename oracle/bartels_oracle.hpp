// FP64 CPU oracle for the tet-mesh hyperelastic path of dilevin/Bartels.
//
// TEST INFRASTRUCTURE ONLY. This header is the checker that the CUDA library in
// bartels_gb300/ is compared against; it is never linked into, called by, or
// used as a fallback for the product path. Only tests/, __graft_entry__.smoke()
// and bench.py's cpu_baseline / --impl reference leg may load it.
//
// It restates the reference's algorithm in plain C++17 (no Eigen), one function
// per reference routine, each citing the reference file:line it follows.
// Storage conventions are the reference's:
//   * V  : nV x 3 double, column-major (all x, then all y, then all z)
//   * E  : nT x 4 int, column-major, 0-based
//   * q  : 3 nV double, interleaved [x0 y0 z0 x1 ...]  (src/linear_tet_neohookean_dq.cpp:15)
//   * dphidX : nT x 12 double, column-major; row t = column-major flatten of the
//     4x3 matrix dphi (include/flatten.h:102-110, src/eval_at_point.cpp:28)
//   * params : nT x 2 double, column-major (one row per tet)
//   * F flatten is column-major [F11 F21 F31 F12 ...].
// Sparse results are returned as CSR of the assembled matrix with duplicates
// summed in element (triplet insertion) order, which is what
// Eigen::SparseMatrix::setFromTriplets does for src/assemble.cpp:57-94.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <numeric>
#include <vector>

namespace oracle {

using std::size_t;

// ----------------------------------------------------------------------------
// small dense helpers (column-major 3x3: a[i + 3*j])
// ----------------------------------------------------------------------------
inline double det3(const double *A) {
  return A[0] * (A[4] * A[8] - A[5] * A[7]) - A[3] * (A[1] * A[8] - A[2] * A[7]) +
         A[6] * (A[1] * A[5] - A[2] * A[4]);
}

// inverse33, include/EigenTypes.h:105-120 (adjugate / determinant; the
// reference builds the cofactor matrix and transposes it in place).
inline void inverse33(double *R, const double *A) {
  auto a = [&](int i, int j) { return A[i + 3 * j]; };
  double det = a(0, 0) * (a(1, 1) * a(2, 2) - a(2, 1) * a(1, 2)) -
               a(0, 1) * (a(1, 0) * a(2, 2) - a(1, 2) * a(2, 0)) +
               a(0, 2) * (a(1, 0) * a(2, 1) - a(1, 1) * a(2, 0));
  double inv = 1.0 / det;
  double C[9];  // cofactor matrix C(i,j)
  C[0 + 3 * 0] = (a(1, 1) * a(2, 2) - a(2, 1) * a(1, 2));
  C[1 + 3 * 0] = -(a(0, 1) * a(2, 2) - a(0, 2) * a(2, 1));
  C[2 + 3 * 0] = (a(0, 1) * a(1, 2) - a(0, 2) * a(1, 1));
  C[0 + 3 * 1] = -(a(1, 0) * a(2, 2) - a(1, 2) * a(2, 0));
  C[1 + 3 * 1] = (a(0, 0) * a(2, 2) - a(0, 2) * a(2, 0));
  C[2 + 3 * 1] = -(a(0, 0) * a(1, 2) - a(1, 0) * a(0, 2));
  C[0 + 3 * 2] = (a(1, 0) * a(2, 1) - a(2, 0) * a(1, 1));
  C[1 + 3 * 2] = -(a(0, 0) * a(2, 1) - a(2, 0) * a(0, 1));
  C[2 + 3 * 2] = (a(0, 0) * a(1, 1) - a(1, 0) * a(0, 1));
  // the reference scales then transposes: R = (C * inv)^T
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) R[i + 3 * j] = C[j + 3 * i] * inv;
}

inline void matmul3(double *C, const double *A, const double *B) {
  double t[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0;
      for (int k = 0; k < 3; ++k) s += A[i + 3 * k] * B[k + 3 * j];
      t[i + 3 * j] = s;
    }
  std::memcpy(C, t, sizeof(t));
}

// cofactor of F, flattened column-major: dJ/dF
inline void cofactor3(double *g, const double *F) {
  auto f = [&](int i, int j) { return F[i + 3 * j]; };
  g[0 + 3 * 0] = f(1, 1) * f(2, 2) - f(1, 2) * f(2, 1);
  g[1 + 3 * 0] = f(0, 2) * f(2, 1) - f(0, 1) * f(2, 2);
  g[2 + 3 * 0] = f(0, 1) * f(1, 2) - f(0, 2) * f(1, 1);
  g[0 + 3 * 1] = f(1, 2) * f(2, 0) - f(1, 0) * f(2, 2);
  g[1 + 3 * 1] = f(0, 0) * f(2, 2) - f(0, 2) * f(2, 0);
  g[2 + 3 * 1] = f(0, 2) * f(1, 0) - f(0, 0) * f(1, 2);
  g[0 + 3 * 2] = f(1, 0) * f(2, 1) - f(1, 1) * f(2, 0);
  g[1 + 3 * 2] = f(0, 1) * f(2, 0) - f(0, 0) * f(2, 1);
  g[2 + 3 * 2] = f(0, 0) * f(1, 1) - f(0, 1) * f(1, 0);
}

inline int levi(int a, int b, int c) {
  if (a == b || b == c || a == c) return 0;
  return ((a == 0 && b == 1) || (a == 1 && b == 2) || (a == 2 && b == 0)) ? 1 : -1;
}

// d^2 det(F) / dF dF, 9x9 column-major-indexed: H[(i+3j) + 9*(k+3l)]
inline void d2det3(double *H, const double *F) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      for (int k = 0; k < 3; ++k)
        for (int l = 0; l < 3; ++l) {
          double v = 0;
          if (i != k && j != l) {
            int m = 3 - i - k, n = 3 - j - l;
            v = levi(i, k, m) * levi(j, l, n) * F[m + 3 * n];
          }
          H[(i + 3 * j) + 9 * (k + 3 * l)] = v;
        }
}

// ----------------------------------------------------------------------------
// kinematics
// ----------------------------------------------------------------------------

// linear_tet_dphi_dX, src/linear_tet_dphi_dX.cpp:10-16: rows 1..3 of the 4x3
// dphi are the inverse of the edge matrix [X1-X0, X2-X0, X3-X0] (edges as
// columns), row 0 is minus the column sums. Output is the column-major flatten
// of dphi (12 doubles), i.e. dphi(a, d) at index a + 4 d.
inline void tet_dphi_dX(double *out12, const double *X0, const double *X1, const double *X2,
                        const double *X3) {
  double Dm[9];
  for (int d = 0; d < 3; ++d) {
    Dm[d + 3 * 0] = X1[d] - X0[d];
    Dm[d + 3 * 1] = X2[d] - X0[d];
    Dm[d + 3 * 2] = X3[d] - X0[d];
  }
  double Di[9];
  inverse33(Di, Dm);
  for (int d = 0; d < 3; ++d) {
    double s = 0;
    for (int a = 1; a < 4; ++a) {
      double v = Di[(a - 1) + 3 * d];  // row a-1 of Dm^{-1}
      out12[a + 4 * d] = v;
      s += v;
    }
    out12[0 + 4 * d] = -s;
  }
}

// Signed tet volume, det[X1-X0, X2-X0, X3-X0] / 6. The reference takes volumes
// from igl::volume (tests/test_constitutive_model.cpp:28); for a positively
// oriented tet both give the same positive value.
inline double tet_volume(const double *X0, const double *X1, const double *X2, const double *X3) {
  double Dm[9];
  for (int d = 0; d < 3; ++d) {
    Dm[d + 3 * 0] = X1[d] - X0[d];
    Dm[d + 3 * 1] = X2[d] - X0[d];
    Dm[d + 3 * 2] = X3[d] - X0[d];
  }
  return det3(Dm) / 6.0;
}

// flatten_multiply_right<Matrix34>(dphidX), include/flatten_multiply.h:44-88:
// dense 9x12 B with vec(F) = B * qe, B[(i+3j), (l+3m)] = (l == i) ? dphi(m, j) : 0.
inline void build_B(double *B /*9x12 col-major*/, const double *dphi12) {
  for (int col = 0; col < 12; ++col)
    for (int row = 0; row < 9; ++row) {
      int i = row % 3, j = row / 3, l = col % 3, m = col / 3;
      B[row + 9 * col] = (l == i) ? dphi12[m + 4 * j] : 0.0;
    }
}

// ----------------------------------------------------------------------------
// constitutive models. params are the reference's per-tet row (2 values).
// ----------------------------------------------------------------------------
enum Model { NEOHOOKEAN = 0, STVK = 1, COROTATIONAL = 2, NEOHOOKEAN_ISOCHORIC = 3, ARAP = 4, LINEAR_ELASTICITY = 5 };

// psi_neohookean_F, src/psi_neohookean_F.cpp:31: C (tr F^T F - 3 - 2 ln J) + D (J-1)^2,
// params = (C, D).
inline double psi_nh(const double *F, const double *p) {
  double J = det3(F), I1 = 0;
  for (int i = 0; i < 9; ++i) I1 += F[i] * F[i];
  return p[0] * (I1 - 3.0 - 2.0 * std::log(J)) + p[1] * (J - 1.0) * (J - 1.0);
}

// dpsi_neohookean_dF, src/dpsi_neohookean_dF.cpp:58-66: 2C (F - cof/J) + 2D (J-1) cof.
inline void dpsi_nh(double *P, const double *F, const double *p) {
  double g[9];
  cofactor3(g, F);
  double J = det3(F);
  for (int i = 0; i < 9; ++i)
    P[i] = p[0] * (2.0 * F[i] - 2.0 * g[i] / J) + 2.0 * p[1] * (J - 1.0) * g[i];
}

// d2psi_neohookean_dF2, src/d2psi_neohookean_dF2.cpp:200-282 in cofactor form:
// 2C I + (2C/J^2 + 2D) g g^T + (2D (J-1) - 2C/J) d2J/dF2, g = cof(F).
inline void d2psi_nh(double *H /*9x9*/, const double *F, const double *p) {
  double g[9], HJ[81];
  cofactor3(g, F);
  d2det3(HJ, F);
  double J = det3(F);
  double a = 2.0 * p[0] / (J * J) + 2.0 * p[1];
  double b = 2.0 * p[1] * (J - 1.0) - 2.0 * p[0] / J;
  for (int r = 0; r < 9; ++r)
    for (int c = 0; c < 9; ++c)
      H[r + 9 * c] = (r == c ? 2.0 * p[0] : 0.0) + a * g[r] * g[c] + b * HJ[r + 9 * c];
}

// Isochoric Neo-Hookean, the reference's earlier law kept as commented-out
// code in src/psi_neohookean_F.cpp:8-14 and src/d2psi_neohookean_dF2.cpp:8-183:
// C (J^{-2/3} tr F^T F - 3) + D (J-1)^2, with J^{2/3} = cbrt(J)^2 (stablePow,
// include/EigenTypes.h:101-103). data/matrices/H_neohookean_coarser_bunny.txt
// was generated with this law.
inline double psi_nh_iso(const double *F, const double *p) {
  double J = det3(F), I1 = 0;
  for (int i = 0; i < 9; ++i) I1 += F[i] * F[i];
  double c = std::cbrt(J);
  return p[0] * (I1 / (c * c) - 3.0) + p[1] * (J - 1.0) * (J - 1.0);
}
inline void dpsi_nh_iso(double *P, const double *F, const double *p) {
  double g[9];
  cofactor3(g, F);
  double J = det3(F), I1 = 0;
  for (int i = 0; i < 9; ++i) I1 += F[i] * F[i];
  double c = std::cbrt(J), Jm23 = 1.0 / (c * c), Jm53 = Jm23 / J;
  for (int i = 0; i < 9; ++i)
    P[i] = p[0] * (2.0 * Jm23 * F[i] - (2.0 / 3.0) * I1 * Jm53 * g[i]) + 2.0 * p[1] * (J - 1.0) * g[i];
}
inline void d2psi_nh_iso(double *H, const double *F, const double *p) {
  double g[9], HJ[81];
  cofactor3(g, F);
  d2det3(HJ, F);
  double J = det3(F), I1 = 0;
  for (int i = 0; i < 9; ++i) I1 += F[i] * F[i];
  double c = std::cbrt(J), Jm23 = 1.0 / (c * c), Jm53 = Jm23 / J, Jm83 = Jm53 / J;
  double C = p[0], D = p[1];
  for (int r = 0; r < 9; ++r)
    for (int k = 0; k < 9; ++k)
      H[r + 9 * k] = (r == k ? 2.0 * C * Jm23 : 0.0) - (4.0 / 3.0) * C * Jm53 * (F[r] * g[k] + g[r] * F[k]) +
                     (10.0 / 9.0) * C * I1 * Jm83 * g[r] * g[k] - (2.0 / 3.0) * C * I1 * Jm53 * HJ[r + 9 * k] +
                     2.0 * D * g[r] * g[k] + 2.0 * D * (J - 1.0) * HJ[r + 9 * k];
}

// psi_stvk_F, src/psi_stvk_F.cpp:11-12, params = (lambda, mu):
// E = (F^T F - I)/2, mu tr(E^2) + lambda/2 tr(E)^2.
inline void green_strain(double *E, const double *F) {
  double C[9], Ft[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) Ft[i + 3 * j] = F[j + 3 * i];
  matmul3(C, Ft, F);
  for (int i = 0; i < 9; ++i) E[i] = 0.5 * (C[i] - ((i % 4) == 0 ? 1.0 : 0.0));
}
inline double psi_stvk(const double *F, const double *p) {
  double E[9], EE[9];
  green_strain(E, F);
  matmul3(EE, E, E);
  double trE = E[0] + E[4] + E[8], trEE = EE[0] + EE[4] + EE[8];
  return p[1] * trEE + 0.5 * p[0] * trE * trE;
}
// dpsi_stvk_dF, src/dpsi_stvk_dF.cpp:25-33: P = F (2 mu E + lambda tr(E) I).
inline void dpsi_stvk(double *P, const double *F, const double *p) {
  double E[9], S[9];
  green_strain(E, F);
  double trE = E[0] + E[4] + E[8];
  for (int i = 0; i < 9; ++i) S[i] = 2.0 * p[1] * E[i] + ((i % 4) == 0 ? p[0] * trE : 0.0);
  matmul3(P, F, S);
}
// d2psi_stvk_dF2, src/d2psi_stvk_dF2.cpp:26-106, as the directional derivative
// dP = dF S + F dS, dS = 2 mu dE + lambda tr(dE) I, dE = (dF^T F + F^T dF)/2.
inline void d2psi_stvk(double *H, const double *F, const double *p) {
  double E[9], S[9];
  green_strain(E, F);
  double trE = E[0] + E[4] + E[8];
  for (int i = 0; i < 9; ++i) S[i] = 2.0 * p[1] * E[i] + ((i % 4) == 0 ? p[0] * trE : 0.0);
  double Ft[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) Ft[i + 3 * j] = F[j + 3 * i];
  for (int c = 0; c < 9; ++c) {
    double dF[9] = {0}, dFt[9], a[9], b[9], dE[9], dS[9], t1[9], t2[9];
    dF[c] = 1.0;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) dFt[i + 3 * j] = dF[j + 3 * i];
    matmul3(a, dFt, F);
    matmul3(b, Ft, dF);
    for (int i = 0; i < 9; ++i) dE[i] = 0.5 * (a[i] + b[i]);
    double trdE = dE[0] + dE[4] + dE[8];
    for (int i = 0; i < 9; ++i) dS[i] = 2.0 * p[1] * dE[i] + ((i % 4) == 0 ? p[0] * trdE : 0.0);
    matmul3(t1, dF, S);
    matmul3(t2, F, dS);
    for (int i = 0; i < 9; ++i) H[i + 9 * c] = t1[i] + t2[i];
  }
}

// --- corotational over singular values -------------------------------------
// psi_corotational_S, src/psi_corotational_S.cpp:8 (params = (lambda, mu)):
// mu sum (s_i - 1)^2 + lambda/2 (sum s_i - 3)^2
inline double psi_corot_S(const double *S, const double *p) {
  double tr = S[0] + S[1] + S[2] - 3.0;
  return p[1] * ((S[0] - 1) * (S[0] - 1) + (S[1] - 1) * (S[1] - 1) + (S[2] - 1) * (S[2] - 1)) +
         0.5 * p[0] * tr * tr;
}
// dpsi_corotational_dS, src/dpsi_corotational_dS.cpp:9-11
inline void dpsi_corot_S(double *d, const double *S, const double *p) {
  double tr = S[0] + S[1] + S[2] - 3.0;
  for (int i = 0; i < 3; ++i) d[i] = 2.0 * p[1] * (S[i] - 1.0) + p[0] * tr;
}
// d2psi_corotational_dS2, src/d2psi_corotational_dS2.cpp:10-12: 2 mu I + lambda 1 1^T
inline void d2psi_corot_S(double *H /*3x3*/, const double *, const double *p) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) H[i + 3 * j] = (i == j ? 2.0 * p[1] : 0.0) + p[0];
}

// Rotation-variant SVD F = U diag(S) V^T with U, V proper rotations,
// |S0| >= |S1| >= |S2|, S0, S1 >= 0 and S2 carrying the sign of det F. This is
// the convention of the reference's SVD (igl::svd3x3, the McAdams et al. 2011
// algorithm, called at src/psi_stretch_F.cpp:18, src/dpsi_stretch_dF.cpp:18,
// src/d2psi_stretch_dF2.cpp:21). Method: cyclic Jacobi on F^T F (V), sort,
// Givens QR of F V (U, S).
inline void svd3(const double *F, double *U, double *S, double *V) {
  double A[9], Ft[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) Ft[i + 3 * j] = F[j + 3 * i];
  matmul3(A, Ft, F);
  for (int i = 0; i < 9; ++i) V[i] = (i % 4 == 0) ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 60; ++sweep) {
    double off = A[3] * A[3] + A[6] * A[6] + A[7] * A[7];
    double dia = A[0] * A[0] + A[4] * A[4] + A[8] * A[8];
    if (off <= 1e-36 * dia || off == 0.0) break;
    const int pr[3][2] = {{0, 1}, {0, 2}, {1, 2}};
    for (auto &pq : pr) {
      int p = pq[0], q = pq[1];
      double apq = A[p + 3 * q];
      if (apq == 0.0) continue;
      double theta = (A[q + 3 * q] - A[p + 3 * p]) / (2.0 * apq);
      double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
      double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
      // A <- J^T A J with J = rotation in (p,q): J(p,p)=c, J(p,q)=s, J(q,p)=-s, J(q,q)=c
      for (int k = 0; k < 3; ++k) {
        double akp = A[k + 3 * p], akq = A[k + 3 * q];
        A[k + 3 * p] = c * akp - s * akq;
        A[k + 3 * q] = s * akp + c * akq;
      }
      for (int k = 0; k < 3; ++k) {
        double apk = A[p + 3 * k], aqk = A[q + 3 * k];
        A[p + 3 * k] = c * apk - s * aqk;
        A[q + 3 * k] = s * apk + c * aqk;
      }
      for (int k = 0; k < 3; ++k) {
        double vkp = V[k + 3 * p], vkq = V[k + 3 * q];
        V[k + 3 * p] = c * vkp - s * vkq;
        V[k + 3 * q] = s * vkp + c * vkq;
      }
    }
  }
  double B[9];
  matmul3(B, F, V);
  double nrm[3];
  for (int j = 0; j < 3; ++j)
    nrm[j] = B[0 + 3 * j] * B[0 + 3 * j] + B[1 + 3 * j] * B[1 + 3 * j] + B[2 + 3 * j] * B[2 + 3 * j];
  // sort columns by descending norm (selection sort on 3 entries)
  for (int a = 0; a < 2; ++a) {
    int m = a;
    for (int b = a + 1; b < 3; ++b)
      if (nrm[b] > nrm[m]) m = b;
    if (m != a) {
      std::swap(nrm[a], nrm[m]);
      for (int k = 0; k < 3; ++k) {
        std::swap(B[k + 3 * a], B[k + 3 * m]);
        std::swap(V[k + 3 * a], V[k + 3 * m]);
      }
    }
  }
  if (det3(V) < 0) {
    for (int k = 0; k < 3; ++k) {
      V[k + 6] = -V[k + 6];
      B[k + 6] = -B[k + 6];
    }
  }
  // Givens QR: R = G3 G2 G1 B, U = (G3 G2 G1)^T
  double Q[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};  // accumulates G (rows)
  auto givens = [&](int i, int k, int col) {
    double a = B[i + 3 * col], b = B[k + 3 * col];
    double r = std::hypot(a, b);
    double c = 1.0, s = 0.0;
    if (r > 0) {
      c = a / r;
      s = b / r;
    }
    for (int j = 0; j < 3; ++j) {
      double bi = B[i + 3 * j], bk = B[k + 3 * j];
      B[i + 3 * j] = c * bi + s * bk;
      B[k + 3 * j] = -s * bi + c * bk;
      double qi = Q[i + 3 * j], qk = Q[k + 3 * j];
      Q[i + 3 * j] = c * qi + s * qk;
      Q[k + 3 * j] = -s * qi + c * qk;
    }
  };
  givens(0, 1, 0);
  givens(0, 2, 0);
  givens(1, 2, 1);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) U[i + 3 * j] = Q[j + 3 * i];
  S[0] = B[0];
  S[1] = B[4];
  S[2] = B[8];
}

// psi_stretch_F with psi_corotational_S, src/psi_stretch_F.cpp:13-21 (signed S).
inline double psi_corot(const double *F, const double *p) {
  double U[9], S[3], V[9];
  svd3(F, U, S, V);
  return psi_corot_S(S, p);
}

// dpsi_stretch_dF with dpsi_corotational_dS, src/dpsi_stretch_dF.cpp:12-45:
// inversion fix (flip negative S when S0 S1 S2 <= -1e-10; reflect U, V if
// det <= 0), then P = U diag(dpsi(S)) V^T flattened column-major.
inline void dpsi_corot(double *P, const double *F, const double *p) {
  double U[9], S[3], V[9];
  svd3(F, U, S, V);
  double det = S[0] * S[1] * S[2];
  if (det <= -1e-10)
    for (int i = 0; i < 3; ++i)
      if (S[i] < 0) S[i] = -S[i];
  if (det3(U) <= 0)
    for (int k = 0; k < 3; ++k) U[k + 6] = -U[k + 6];
  if (det3(V) <= 0)
    for (int k = 0; k < 3; ++k) V[k + 6] = -V[k + 6];
  double d[3];
  dpsi_corot_S(d, S, p);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double s = 0;
      for (int k = 0; k < 3; ++k) s += U[i + 3 * k] * d[k] * V[j + 3 * k];
      P[i + 3 * j] = s;
    }
}

// Exact Hessian of psi(S(F)) in column-major indexing from the eigen-system of
// a stretch-based energy (scaling block d2psi/dS2, twist (dpsi_i + dpsi_j) /
// (s_i + s_j), flip (dpsi_i - dpsi_j) / (s_i - s_j)). Mathematically identical
// to the dU/dS/dV route of src/dsvd.cpp:8-56 + src/d2psi_stretch_dF2.cpp:30-45
// wherever the singular values are distinct. At repeated singular values the
// reference perturbs F randomly (src/d2psi_stretch_dF2.cpp:25-28); here the
// exact limit is used instead (flip = d2psi_ii - d2psi_ij = 2 mu). Where the
// reference's dsvd zeroes the rotation rates (|s_j^2 - s_i^2| < 1e-8 with
// distinct s, src/dsvd.cpp:21-23) the pair contributes nothing, as there.
inline void d2psi_corot_exact_cm(double *H, const double *F, const double *p) {
  double U[9], S[3], V[9];
  svd3(F, U, S, V);
  double d[3], dd[9];
  dpsi_corot_S(d, S, p);
  d2psi_corot_S(dd, S, p);
  std::fill(H, H + 81, 0.0);
  // scaling modes: vec(u_i v_i^T)
  double D[3][9];
  for (int i = 0; i < 3; ++i)
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) D[i][r + 3 * c] = U[r + 3 * i] * V[c + 3 * i];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      for (int a = 0; a < 9; ++a)
        for (int b = 0; b < 9; ++b) H[a + 9 * b] += dd[i + 3 * j] * D[i][a] * D[j][b];
  const int pr[3][2] = {{0, 1}, {0, 2}, {1, 2}};
  const double is2 = 1.0 / std::sqrt(2.0);
  for (auto &ij : pr) {
    int i = ij[0], j = ij[1];
    double lt = 0.0, lf = 0.0;
    bool repeated = std::fabs(S[i] - S[j]) < 1e-5;
    bool stalled = !repeated && std::fabs(S[j] * S[j] - S[i] * S[i]) < 1e-8;
    if (!stalled) {
      lf = repeated ? (dd[i + 3 * i] - dd[i + 3 * j]) : (d[i] - d[j]) / (S[i] - S[j]);
      double den = S[i] + S[j];
      lt = (den != 0.0) ? (d[i] + d[j]) / den : 0.0;
    }
    double T[9], Fl[9];
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) {
        double a = U[r + 3 * i] * V[c + 3 * j], b = U[r + 3 * j] * V[c + 3 * i];
        T[r + 3 * c] = (a - b) * is2;
        Fl[r + 3 * c] = (a + b) * is2;
      }
    for (int a = 0; a < 9; ++a)
      for (int b = 0; b < 9; ++b) H[a + 9 * b] += lt * T[a] * T[b] + lf * Fl[a] * Fl[b];
  }
}

// The reference's d2psi_stretch_dF2 (src/d2psi_stretch_dF2.cpp:37-45) stores
// d P / d F(r,s) in row 3r+s and flattens P row-major (transposeInPlace + Map),
// while B (include/flatten_multiply.h) indexes F column-major. The matrix the
// reference contracts with B is therefore Pi H Pi, Pi the row/column-major
// index swap. layout_reference = true reproduces that; false gives the exact
// column-major Hessian.
inline void d2psi_corot(double *H, const double *F, const double *p, bool layout_reference) {
  double Hc[81];
  d2psi_corot_exact_cm(Hc, F, p);
  if (!layout_reference) {
    std::memcpy(H, Hc, sizeof(Hc));
    return;
  }
  auto pi = [](int c) { return 3 * (c % 3) + c / 3; };
  for (int a = 0; a < 9; ++a)
    for (int b = 0; b < 9; ++b) H[pi(a) + 9 * pi(b)] = Hc[a + 9 * b];
}

// Literal transcription of the reference's dU/dS/dV route (src/dsvd.cpp:8-56,
// src/d2psi_stretch_dF2.cpp:30-45, without the random perturbation). Used only
// by tests to show that d2psi_corot(layout_reference=true) equals it whenever
// the singular values are distinct.
inline void d2psi_corot_dsvd_literal(double *H, const double *F, const double *p) {
  double U[9], S[3], V[9];
  svd3(F, U, S, V);
  double Pl[3], P2[9];
  dpsi_corot_S(Pl, S, p);
  d2psi_corot_S(P2, S, p);
  double tol = 1e-8;
  double d01 = S[1] * S[1] - S[0] * S[0], d02 = S[2] * S[2] - S[0] * S[0],
         d12 = S[2] * S[2] - S[1] * S[1];
  d01 = std::fabs(d01) < tol ? 0.0 : 1.0 / d01;
  d02 = std::fabs(d02) < tol ? 0.0 : 1.0 / d02;
  d12 = std::fabs(d12) < tol ? 0.0 : 1.0 / d12;
  for (int r = 0; r < 3; ++r)
    for (int s = 0; s < 3; ++s) {
      double UVT[9];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) UVT[i + 3 * j] = U[r + 3 * i] * V[s + 3 * j];
      double dS[3] = {UVT[0], UVT[4], UVT[8]};
      for (int i = 0; i < 3; ++i) UVT[i + 3 * i] = 0.0;
      double tmp[9];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) tmp[i + 3 * j] = S[i] * UVT[i + 3 * j] + UVT[j + 3 * i] * S[j];
      double w01 = tmp[0 + 3] * d01, w02 = tmp[0 + 6] * d02, w12 = tmp[1 + 6] * d12;
      double Om[9] = {0, -w01, -w02, w01, 0, -w12, w02, w12, 0};
      double dV[9];
      matmul3(dV, V, Om);
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) tmp[i + 3 * j] = UVT[i + 3 * j] * S[j] + S[i] * UVT[j + 3 * i];
      w01 = tmp[0 + 3] * d01;
      w02 = tmp[0 + 6] * d02;
      w12 = tmp[1 + 6] * d12;
      double Om2[9] = {0, -w01, -w02, w01, 0, -w12, w02, w12, 0};
      double dU[9];
      matmul3(dU, U, Om2);
      double Pv[3];
      for (int i = 0; i < 3; ++i) Pv[i] = P2[i + 0] * dS[0] + P2[i + 3] * dS[1] + P2[i + 6] * dS[2];
      double R[9];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          double v = 0;
          for (int k = 0; k < 3; ++k)
            v += dU[i + 3 * k] * Pl[k] * V[j + 3 * k] + U[i + 3 * k] * Pl[k] * dV[j + 3 * k] +
                 U[i + 3 * k] * Pv[k] * V[j + 3 * k];
          R[i + 3 * j] = v;
        }
      // row 3r+s, columns row-major over R
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) H[(3 * r + s) + 9 * (3 * i + j)] = R[i + 3 * j];
    }
}

// --- ARAP -------------------------------------------------------------------
// psi_arap_S, src/psi_arap_S.cpp:8-11: k sum (s_i - 1)^2 (k = params(0));
// dpsi_arap_dS, src/dpsi_arap_dS.cpp:8-10: 2 k (s_i - 1); d2psi_arap_dS2,
// src/d2psi_arap_dS2.cpp:8-9: 2 k I. linear_tet_arap_{q,dq,dq2}
// (src/linear_tet_arap_q.cpp:12, _dq.cpp:13-14, _dq2.cpp:12-14) pass these
// through the same stretch routines as the corotational model, whose
// S-functions with (lambda, mu) = (0, k) are exactly these; so ARAP is
// evaluated as the corotational stretch energy with lambda = 0, mu = k.
inline void arap_params(double *pc, const double *p) {
  pc[0] = 0.0;
  pc[1] = p[0];
}
inline double psi_arap(const double *F, const double *p) {
  double pc[2];
  arap_params(pc, p);
  return psi_corot(F, pc);
}
inline void dpsi_arap(double *P, const double *F, const double *p) {
  double pc[2];
  arap_params(pc, p);
  dpsi_corot(P, F, pc);
}
inline void d2psi_arap(double *H, const double *F, const double *p, bool layout_reference) {
  double pc[2];
  arap_params(pc, p);
  d2psi_corot(H, F, pc, layout_reference);
}

// --- linear elasticity --------------------------------------------------------
// linear_tet_linear_elasticity_dq2, src/linear_tet_linear_elasticity_dq2.cpp:8-25:
// B6 = P2 B with P2 (6x9) picking [F11, F22, F33, F32 + F23, F31 + F13,
// F21 + F12] from vec(F) (column-major), C from
// src/d2psi_linear_elasticity_de2.cpp:8-24 (params = Young's modulus, Poisson
// ratio), K = B6^T C B6 vol. In F space: psi = 1/2 (P2 f)^T C (P2 f),
// dpsi = P2^T C P2 f (src/linear_tet_linear_elasticity_dq.cpp:17-21 with its
// 6/9 size mismatch resolved), d2psi = P2^T C P2.
inline void le_C(double *C /*6x6 col-major*/, const double *p) {
  for (int i = 0; i < 36; ++i) C[i] = 0.0;
  const double YM = p[0], nu = p[1];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) C[i + 6 * j] = (i == j) ? 1.0 - nu : nu;
  for (int i = 3; i < 6; ++i) C[i + 6 * i] = 0.5 * (1.0 - 2.0 * nu);
  const double s = YM / ((1.0 + nu) * (1.0 - 2.0 * nu));
  for (int i = 0; i < 36; ++i) C[i] *= s;
}
inline void le_P2(double *P /*6x9 col-major*/) {
  for (int i = 0; i < 54; ++i) P[i] = 0.0;
  const int rows[9][2] = {{0, -1}, {5, -1}, {4, -1}, {5, -1}, {1, -1}, {3, -1}, {4, -1}, {3, -1}, {2, -1}};
  // column c of vec(F) contributes to Voigt row rows[c][0]
  for (int c = 0; c < 9; ++c) P[rows[c][0] + 6 * c] = 1.0;
}
inline void le_CP(double *CP /*6x9*/, const double *p) {
  double C[36], P[54];
  le_C(C, p);
  le_P2(P);
  for (int i = 0; i < 6; ++i)
    for (int c = 0; c < 9; ++c) {
      double acc = 0.0;
      for (int k = 0; k < 6; ++k) acc += C[i + 6 * k] * P[k + 6 * c];
      CP[i + 6 * c] = acc;
    }
}
inline double psi_le(const double *F, const double *p) {
  double P[54], C[36], e[6] = {0, 0, 0, 0, 0, 0};
  le_P2(P);
  le_C(C, p);
  for (int i = 0; i < 6; ++i)
    for (int c = 0; c < 9; ++c) e[i] += P[i + 6 * c] * F[c];
  double acc = 0.0;
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) acc += e[i] * C[i + 6 * j] * e[j];
  return 0.5 * acc;
}
inline void dpsi_le(double *Pk, const double *F, const double *p) {
  double P[54], CP[54];
  le_P2(P);
  le_CP(CP, p);
  double s[6] = {0, 0, 0, 0, 0, 0};
  for (int i = 0; i < 6; ++i)
    for (int c = 0; c < 9; ++c) s[i] += CP[i + 6 * c] * F[c];
  for (int c = 0; c < 9; ++c) {
    double acc = 0.0;
    for (int i = 0; i < 6; ++i) acc += P[i + 6 * c] * s[i];
    Pk[c] = acc;
  }
}
inline void d2psi_le(double *H /*9x9 col-major*/, const double *p) {
  double P[54], CP[54];
  le_P2(P);
  le_CP(CP, p);
  for (int a = 0; a < 9; ++a)
    for (int b = 0; b < 9; ++b) {
      double acc = 0.0;
      for (int i = 0; i < 6; ++i) acc += P[i + 6 * a] * CP[i + 6 * b];
      H[a + 9 * b] = acc;
    }
}

// ----------------------------------------------------------------------------
// per-element energy / gradient / Hessian: linear_tet_{model}_{q,dq,dq2}
// (src/linear_tet_neohookean_q.cpp:9-16, _dq.cpp:11-20, _dq2.cpp:12-21 and the
// StVK / corotational twins): F = unflatten(B qe); q = psi vol; dq = B^T dpsi vol;
// dq2 = B^T d2psi B vol.
// ----------------------------------------------------------------------------
struct ElementFlags {
  bool corot_layout_reference = true;
};

inline void element_F(double *F, const double *B, const double *qe) {
  for (int r = 0; r < 9; ++r) {
    double s = 0;
    for (int c = 0; c < 12; ++c) s += B[r + 9 * c] * qe[c];
    F[r] = s;
  }
}

inline double model_psi(int model, const double *F, const double *p) {
  switch (model) {
    case NEOHOOKEAN: return psi_nh(F, p);
    case STVK: return psi_stvk(F, p);
    case NEOHOOKEAN_ISOCHORIC: return psi_nh_iso(F, p);
    case ARAP: return psi_arap(F, p);
    case LINEAR_ELASTICITY: return psi_le(F, p);
    default: return psi_corot(F, p);
  }
}
inline void model_dpsi(int model, double *P, const double *F, const double *p) {
  switch (model) {
    case NEOHOOKEAN: dpsi_nh(P, F, p); break;
    case STVK: dpsi_stvk(P, F, p); break;
    case NEOHOOKEAN_ISOCHORIC: dpsi_nh_iso(P, F, p); break;
    case ARAP: dpsi_arap(P, F, p); break;
    case LINEAR_ELASTICITY: dpsi_le(P, F, p); break;
    default: dpsi_corot(P, F, p); break;
  }
}
inline void model_d2psi(int model, double *H, const double *F, const double *p, const ElementFlags &fl) {
  switch (model) {
    case NEOHOOKEAN: d2psi_nh(H, F, p); break;
    case STVK: d2psi_stvk(H, F, p); break;
    case NEOHOOKEAN_ISOCHORIC: d2psi_nh_iso(H, F, p); break;
    case ARAP: d2psi_arap(H, F, p, fl.corot_layout_reference); break;
    case LINEAR_ELASTICITY: d2psi_le(H, p); break;
    default: d2psi_corot(H, F, p, fl.corot_layout_reference); break;
  }
}

inline double element_q(int model, const double *qe, const double *dphi12, const double *p, double vol) {
  double B[108], F[9];
  build_B(B, dphi12);
  element_F(F, B, qe);
  return model_psi(model, F, p) * vol;
}
inline void element_dq(int model, double *g12, const double *qe, const double *dphi12, const double *p,
                       double vol) {
  double B[108], F[9], P[9];
  build_B(B, dphi12);
  element_F(F, B, qe);
  model_dpsi(model, P, F, p);
  for (int c = 0; c < 12; ++c) {
    double s = 0;
    for (int r = 0; r < 9; ++r) s += B[r + 9 * c] * P[r];
    g12[c] = s * vol;
  }
}
inline void element_dq2(int model, double *K /*12x12 col-major*/, const double *qe, const double *dphi12,
                        const double *p, double vol, const ElementFlags &fl) {
  double B[108], F[9], H[81], HB[108];
  build_B(B, dphi12);
  element_F(F, B, qe);
  model_d2psi(model, H, F, p, fl);
  for (int r = 0; r < 9; ++r)
    for (int c = 0; c < 12; ++c) {
      double s = 0;
      for (int k = 0; k < 9; ++k) s += H[r + 9 * k] * B[k + 9 * c];
      HB[r + 9 * c] = s;
    }
  for (int a = 0; a < 12; ++a)
    for (int b = 0; b < 12; ++b) {
      double s = 0;
      for (int r = 0; r < 9; ++r) s += B[r + 9 * a] * HB[r + 9 * b];
      K[a + 12 * b] = s * vol;
    }
}

// simple_psd_fix, src/simple_psd_fix.cpp:9-19: full symmetric eigen-decomposition
// (reference: Eigen::SelfAdjointEigenSolver, reading the lower triangle), every
// eigenvalue below tol set to tol, A = Q diag Q^T. Cyclic Jacobi here.
inline void psd_fix(double *A, int n, double tol) {
  double Mbuf[144], Qbuf[144];
  std::vector<double> Mv, Qv;
  double *M = Mbuf, *Q = Qbuf;
  if (n > 12) {
    Mv.resize(n * n);
    Qv.resize(n * n);
    M = Mv.data();
    Q = Qv.data();
  }
  for (int i = 0; i < n * n; ++i) Q[i] = 0.0;
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) M[i + n * j] = (i >= j) ? A[i + n * j] : A[j + n * i];
  for (int i = 0; i < n; ++i) Q[i + n * i] = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0, tot = 0;
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        tot += M[i + n * j] * M[i + n * j];
        if (i != j) off += M[i + n * j] * M[i + n * j];
      }
    if (off <= 1e-32 * tot || off == 0.0) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        double apq = M[p + n * q];
        if (apq == 0.0) continue;
        double theta = (M[q + n * q] - M[p + n * p]) / (2.0 * apq);
        double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; ++k) {
          double mkp = M[k + n * p], mkq = M[k + n * q];
          M[k + n * p] = c * mkp - s * mkq;
          M[k + n * q] = s * mkp + c * mkq;
        }
        for (int k = 0; k < n; ++k) {
          double mpk = M[p + n * k], mqk = M[q + n * k];
          M[p + n * k] = c * mpk - s * mqk;
          M[q + n * k] = s * mpk + c * mqk;
        }
        for (int k = 0; k < n; ++k) {
          double qkp = Q[k + n * p], qkq = Q[k + n * q];
          Q[k + n * p] = c * qkp - s * qkq;
          Q[k + n * q] = s * qkp + c * qkq;
        }
      }
  }
  std::vector<double> lamv(n > 144 ? n : 0);
  double lamb[144];
  double *lam = n > 144 ? lamv.data() : lamb;
  for (int i = 0; i < n; ++i) lam[i] = std::max(M[i + n * i], tol);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      double s = 0;
      for (int k = 0; k < n; ++k) s += Q[i + n * k] * lam[k] * Q[j + n * k];
      A[i + n * j] = s;
    }
}

// The same projection with the method class of Eigen's SelfAdjointEigenSolver
// (Householder tridiagonalisation, then implicit-shift QL iterations on the
// tridiagonal matrix with the rotations accumulated into the eigenvectors;
// Golub & Van Loan, Matrix Computations, 8.3; Wilkinson & Reinsch's tred2 /
// tql2): O(n^3) with a small constant where cyclic Jacobi takes many sweeps.
// Used by the timed CPU baseline so that its cost per element is that of a
// production eigen-solver; the parity checks keep psd_fix above. n <= 12.
// Returns false if the QL iteration did not converge (A left unchanged).
inline bool psd_fix_ql(double *A, int n, double tol) {
  double Z[144], d[12], e[12];
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) Z[i + n * j] = (i >= j) ? A[i + n * j] : A[j + n * i];
  // Householder reflections H_k = I - 2 v v^T zero column k below the
  // subdiagonal; Q = H_0 H_1 ... is accumulated separately.
  double Q[144];
  for (int i = 0; i < n * n; ++i) Q[i] = 0.0;
  for (int i = 0; i < n; ++i) Q[i + n * i] = 1.0;
  for (int k = 0; k + 2 < n; ++k) {
    double v[12], nx = 0.0;
    for (int i = k + 1; i < n; ++i) nx += Z[i + n * k] * Z[i + n * k];
    nx = std::sqrt(nx);
    if (nx == 0.0) continue;
    const double x0 = Z[(k + 1) + n * k];
    const double alpha = x0 >= 0.0 ? -nx : nx;
    double nv = 0.0;
    for (int i = k + 1; i < n; ++i) {
      v[i] = Z[i + n * k] - (i == k + 1 ? alpha : 0.0);
      nv += v[i] * v[i];
    }
    nv = std::sqrt(nv);
    if (nv == 0.0) continue;
    for (int i = k + 1; i < n; ++i) v[i] /= nv;
    // trailing block: A22 <- A22 - 2 v w^T - 2 w v^T, w = p - (v^T p) v, p = A22 v
    double p[12], vp = 0.0;
    for (int i = k + 1; i < n; ++i) {
      double s = 0.0;
      for (int j = k + 1; j < n; ++j) s += Z[i + n * j] * v[j];
      p[i] = s;
      vp += v[i] * s;
    }
    for (int i = k + 1; i < n; ++i) p[i] -= vp * v[i];
    for (int i = k + 1; i < n; ++i)
      for (int j = k + 1; j < n; ++j) Z[i + n * j] -= 2.0 * (v[i] * p[j] + p[i] * v[j]);
    Z[(k + 1) + n * k] = Z[k + n * (k + 1)] = alpha;
    for (int i = k + 2; i < n; ++i) Z[i + n * k] = Z[k + n * i] = 0.0;
    for (int r = 0; r < n; ++r) {  // Q <- Q H_k
      double s = 0.0;
      for (int i = k + 1; i < n; ++i) s += Q[r + n * i] * v[i];
      for (int i = k + 1; i < n; ++i) Q[r + n * i] -= 2.0 * s * v[i];
    }
  }
  for (int i = 0; i < n; ++i) d[i] = Z[i + n * i];
  for (int i = 0; i + 1 < n; ++i) e[i] = Z[(i + 1) + n * i];
  e[n - 1] = 0.0;
  // implicit QL with Wilkinson-type shifts; rotations applied to Q's columns
  for (int l = 0; l < n; ++l) {
    for (int iter = 0;; ++iter) {
      int m = l;
      for (; m + 1 < n; ++m) {
        const double dd = std::fabs(d[m]) + std::fabs(d[m + 1]);
        if (std::fabs(e[m]) + dd == dd) break;  // e[m] below the rounding of d
      }
      if (m == l) break;
      if (iter == 60) return false;
      double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
      double r = std::hypot(g, 1.0);
      g = d[m] - d[l] + e[l] / (g + (g >= 0.0 ? r : -r));
      double s = 1.0, c = 1.0, pp = 0.0;
      int i = m - 1;
      for (; i >= l; --i) {
        const double f = s * e[i], b = c * e[i];
        r = std::hypot(f, g);
        e[i + 1] = r;
        if (r == 0.0) {  // split: restart the sweep on the smaller block
          d[i + 1] -= pp;
          e[m] = 0.0;
          break;
        }
        s = f / r;
        c = g / r;
        g = d[i + 1] - pp;
        r = (d[i] - g) * s + 2.0 * c * b;
        pp = s * r;
        d[i + 1] = g + pp;
        g = c * r - b;
        for (int k = 0; k < n; ++k) {
          const double zi = Q[k + n * i], zi1 = Q[k + n * (i + 1)];
          Q[k + n * (i + 1)] = s * zi + c * zi1;
          Q[k + n * i] = c * zi - s * zi1;
        }
      }
      if (r == 0.0 && i >= l) continue;
      d[l] -= pp;
      e[l] = g;
      e[m] = 0.0;
    }
  }
  for (int i = 0; i < n; ++i) d[i] = std::max(d[i], tol);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j <= i; ++j) {
      double s = 0.0;
      for (int k = 0; k < n; ++k) s += Q[i + n * k] * d[k] * Q[j + n * k];
      A[i + n * j] = A[j + n * i] = s;
    }
  return true;
}

// ----------------------------------------------------------------------------
// assembly, src/assemble.cpp
// ----------------------------------------------------------------------------
struct CSR {
  int n = 0;
  std::vector<int> row_ptr, col;
  std::vector<double> val;
};

struct Triplet {
  int r, c;
  double v;
};

// setFromTriplets semantics: duplicates summed in insertion order, indices sorted.
inline void triplets_to_csr(CSR &out, int n, const std::vector<Triplet> &trip) {
  out.n = n;
  std::vector<int> cnt(n + 1, 0);
  for (auto &t : trip) cnt[t.r + 1]++;
  for (int i = 0; i < n; ++i) cnt[i + 1] += cnt[i];
  std::vector<int> order(trip.size());
  std::vector<int> pos(cnt.begin(), cnt.end() - 1);
  for (size_t k = 0; k < trip.size(); ++k) order[pos[trip[k].r]++] = (int)k;  // stable by row
  out.row_ptr.assign(n + 1, 0);
  out.col.clear();
  out.val.clear();
  for (int i = 0; i < n; ++i) {
    auto b = order.begin() + cnt[i], e = order.begin() + cnt[i + 1];
    std::stable_sort(b, e, [&](int x, int y) { return trip[x].c < trip[y].c; });
    int last = -1;
    for (auto it = b; it != e; ++it) {
      const Triplet &t = trip[*it];
      if (t.c == last) {
        out.val.back() += t.v;
      } else {
        out.col.push_back(t.c);
        out.val.push_back(t.v);
        last = t.c;
      }
    }
    out.row_ptr[i + 1] = (int)out.col.size();
  }
}

// matrix assembly of 12x12 element blocks with the reference's triplet order
// (src/assemble.cpp:68-74: column jj outer, row ii inner).
template <class ElemFn>
inline void assemble_matrix(CSR &out, int nV, int nT, const int *E, ElemFn fn) {
  std::vector<Triplet> trip;
  trip.reserve((size_t)nT * 144);
  double K[144];
  for (int ie = 0; ie < nT; ++ie) {
    fn(ie, K);
    for (int jj = 0; jj < 12; ++jj)
      for (int ii = 0; ii < 12; ++ii)
        trip.push_back({3 * E[ie + (size_t)nT * (ii / 3)] + ii % 3, 3 * E[ie + (size_t)nT * (jj / 3)] + jj % 3,
                        K[ii + 12 * jj]});
  }
  triplets_to_csr(out, 3 * nV, trip);
}

inline void gather_qe(double *qe, const double *q, const int *E, int nT, int ie) {
  for (int a = 0; a < 4; ++a) {
    int v = E[ie + (size_t)nT * a];
    for (int d = 0; d < 3; ++d) qe[3 * a + d] = q[3 * v + d];
  }
}
inline void row_of(double *out, const double *M, int nrows, int ncols, int ie) {
  for (int c = 0; c < ncols; ++c) out[c] = M[ie + (size_t)nrows * c];
}

}  // namespace oracle
