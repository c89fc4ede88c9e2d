// Element math of the tet-mesh hot path, written once for device and host.
//
// Compiled by nvcc into the CUDA kernels, and by g++ into a CPU unit-test
// harness that checks these laws against the FP64 oracle. Nothing here
// allocates or branches on the host; all arrays are small and fixed-size.
//
// Conventions: 3x3 matrices are column-major (m[i + 3 j]); F indexes the
// deformation gradient with rows = spatial components, columns = material
// directions, as in the reference's column-major flatten. phi_a is the
// gradient of shape function a (row a of the reference's 4x3 dphidX).
#pragma once

#ifdef __CUDACC__
#define BT_HD __host__ __device__ __forceinline__
#define BT_HD_NOINLINE __host__ __device__ __noinline__
#else
#define BT_HD inline
#define BT_HD_NOINLINE
#include <cmath>
#endif

namespace bartels {

#ifdef __CUDACC__
BT_HD float bt_sqrt(float x) { return sqrtf(x); }
BT_HD double bt_sqrt(double x) { return sqrt(x); }
BT_HD float bt_log(float x) { return logf(x); }
BT_HD double bt_log(double x) { return log(x); }
BT_HD float bt_cbrt(float x) { return cbrtf(x); }
BT_HD double bt_cbrt(double x) { return cbrt(x); }
BT_HD float bt_abs(float x) { return fabsf(x); }
BT_HD double bt_abs(double x) { return fabs(x); }
#else
BT_HD float bt_sqrt(float x) { return std::sqrt(x); }
BT_HD double bt_sqrt(double x) { return std::sqrt(x); }
BT_HD float bt_log(float x) { return std::log(x); }
BT_HD double bt_log(double x) { return std::log(x); }
BT_HD float bt_cbrt(float x) { return std::cbrt(x); }
BT_HD double bt_cbrt(double x) { return std::cbrt(x); }
BT_HD float bt_abs(float x) { return std::fabs(x); }
BT_HD double bt_abs(double x) { return std::fabs(x); }
#endif

enum { MODEL_NH = 0, MODEL_STVK = 1, MODEL_COROT = 2, MODEL_NH_ISO = 3, MODEL_ARAP = 4, MODEL_LE = 5 };

template <class T>
BT_HD T det3(const T *A) {
  return A[0] * (A[4] * A[8] - A[5] * A[7]) - A[3] * (A[1] * A[8] - A[2] * A[7]) +
         A[6] * (A[1] * A[5] - A[2] * A[4]);
}

// cofactor matrix G = dJ/dF (column-major)
template <class T>
BT_HD void cof3(T *G, const T *F) {
  G[0] = F[4] * F[8] - F[7] * F[5];
  G[1] = F[6] * F[5] - F[3] * F[8];
  G[2] = F[3] * F[7] - F[6] * F[4];
  G[3] = F[7] * F[2] - F[1] * F[8];
  G[4] = F[0] * F[8] - F[6] * F[2];
  G[5] = F[6] * F[1] - F[0] * F[7];
  G[6] = F[1] * F[5] - F[4] * F[2];
  G[7] = F[3] * F[2] - F[0] * F[5];
  G[8] = F[0] * F[4] - F[3] * F[1];
}

// y = A x
template <class T>
BT_HD void mv3(T *y, const T *A, const T *x) {
  y[0] = A[0] * x[0] + A[3] * x[1] + A[6] * x[2];
  y[1] = A[1] * x[0] + A[4] * x[1] + A[7] * x[2];
  y[2] = A[2] * x[0] + A[5] * x[1] + A[8] * x[2];
}
// y = A^T x
template <class T>
BT_HD void mtv3(T *y, const T *A, const T *x) {
  y[0] = A[0] * x[0] + A[1] * x[1] + A[2] * x[2];
  y[1] = A[3] * x[0] + A[4] * x[1] + A[5] * x[2];
  y[2] = A[6] * x[0] + A[7] * x[1] + A[8] * x[2];
}
template <class T>
BT_HD T dot3(const T *a, const T *b) {
  return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}
template <class T>
BT_HD void cross3(T *c, const T *a, const T *b) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}

// Deformation gradient F = F0 + sum_{a=1..3} (x_a - x_0) phi_a^T, where F0 is
// the identity when x holds displacements from a rest shape consistent with
// phi, and zero when x holds positions.
template <class T>
BT_HD void def_grad(T *F, const T *x0, const T *x1, const T *x2, const T *x3, const T *dphi9, bool add_identity) {
  T d1[3] = {x1[0] - x0[0], x1[1] - x0[1], x1[2] - x0[2]};
  T d2[3] = {x2[0] - x0[0], x2[1] - x0[1], x2[2] - x0[2]};
  T d3[3] = {x3[0] - x0[0], x3[1] - x0[1], x3[2] - x0[2]};
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      F[i + 3 * j] = d1[i] * dphi9[0 + j] + d2[i] * dphi9[3 + j] + d3[i] * dphi9[6 + j] +
                     ((add_identity && i == j) ? T(1) : T(0));
}

// ----------------------------------------------------------------------------
// Hessian block laws: block(pa, pb, K) returns the 3x3 block (row-major K[k*3+l])
// K_ab[k][l] = sum_{i,j} pa_i pb_j d2psi/dF(k,i)dF(l,j), with psi already scaled
// by the tet volume (pv = vol * params). All laws are bilinear in (pa, pb).
// ----------------------------------------------------------------------------

// Neo-Hookean, psi = C (I1 - 3 - 2 ln J) + D (J-1)^2 (src/psi_neohookean_F.cpp:31).
// d2psi = 2C I + (2C/J^2 + 2D) g g^T + (2D (J-1) - 2C/J) d2J, g = cof F, so
// K_ab = 2C (pa.pb) I + ca (G pa)(G pb)^T + cb [F (pa x pb)]_x.
template <class T>
struct LawNH {
  T F[9], G[9], c2, ca, cb;
  BT_HD LawNH(const T *F_, const T *pv) {
    for (int i = 0; i < 9; ++i) F[i] = F_[i];
    cof3(G, F);
    T J = F[0] * G[0] + F[1] * G[1] + F[2] * G[2];
    T C = pv[0], D = pv[1];
    c2 = T(2) * C;
    ca = T(2) * C / (J * J) + T(2) * D;
    cb = T(2) * D * (J - T(1)) - T(2) * C / J;
  }
  BT_HD void block(const T *pa, const T *pb, T *K) const {
    T ga[3], gb[3], c[3], w[3];
    mv3(ga, G, pa);
    mv3(gb, G, pb);
    cross3(c, pa, pb);
    mv3(w, F, c);
    T d = c2 * dot3(pa, pb);
    for (int k = 0; k < 3; ++k)
      for (int l = 0; l < 3; ++l) K[3 * k + l] = ca * ga[k] * gb[l] + (k == l ? d : T(0));
    K[1] += cb * w[2];
    K[2] -= cb * w[1];
    K[3] -= cb * w[2];
    K[5] += cb * w[0];
    K[6] += cb * w[1];
    K[7] -= cb * w[0];
  }
};

// Isochoric Neo-Hookean, psi = C (J^{-2/3} I1 - 3) + D (J-1)^2 (the
// reference's earlier law, src/psi_neohookean_F.cpp:8-14):
// d2psi = 2C J^-2/3 I - 4/3 C J^-5/3 (F g^T + g F^T) + (10/9 C I1 J^-8/3 + 2D) g g^T
//       + (2D (J-1) - 2/3 C I1 J^-5/3) d2J.
template <class T>
struct LawNHIso {
  T F[9], G[9], a0, a1, a2, a3;
  BT_HD LawNHIso(const T *F_, const T *pv) {
    for (int i = 0; i < 9; ++i) F[i] = F_[i];
    cof3(G, F);
    T J = F[0] * G[0] + F[1] * G[1] + F[2] * G[2];
    T I1 = T(0);
    for (int i = 0; i < 9; ++i) I1 += F[i] * F[i];
    T c = bt_cbrt(J), Jm23 = T(1) / (c * c), Jm53 = Jm23 / J, Jm83 = Jm53 / J;
    T C = pv[0], D = pv[1];
    a0 = T(2) * C * Jm23;
    a1 = -T(4) / T(3) * C * Jm53;
    a2 = T(10) / T(9) * C * I1 * Jm83 + T(2) * D;
    a3 = T(2) * D * (J - T(1)) - T(2) / T(3) * C * I1 * Jm53;
  }
  BT_HD void block(const T *pa, const T *pb, T *K) const {
    T ga[3], gb[3], fa[3], fb[3], c[3], w[3];
    mv3(ga, G, pa);
    mv3(gb, G, pb);
    mv3(fa, F, pa);
    mv3(fb, F, pb);
    cross3(c, pa, pb);
    mv3(w, F, c);
    T d = a0 * dot3(pa, pb);
    for (int k = 0; k < 3; ++k)
      for (int l = 0; l < 3; ++l)
        K[3 * k + l] = a1 * (fa[k] * gb[l] + ga[k] * fb[l]) + a2 * ga[k] * gb[l] + (k == l ? d : T(0));
    K[1] += a3 * w[2];
    K[2] -= a3 * w[1];
    K[3] -= a3 * w[2];
    K[5] += a3 * w[0];
    K[6] += a3 * w[1];
    K[7] -= a3 * w[0];
  }
};

// StVK, psi = mu tr(E^2) + lambda/2 tr(E)^2, E = (F^T F - I)/2, pv = vol (lambda, mu)
// (src/psi_stvk_F.cpp:11-12). From dP = dF S + F dS, S = 2 mu E + lambda tr(E) I:
// K_ab = (pa . S pb) I + mu ((F pb)(F pa)^T + (pa . pb) F F^T) + lambda (F pa)(F pb)^T.
template <class T>
struct LawStVK {
  T F[9], S[9], FFt[6], lam, mu;
  BT_HD LawStVK(const T *F_, const T *pv) {
    for (int i = 0; i < 9; ++i) F[i] = F_[i];
    lam = pv[0];
    mu = pv[1];
    T C[9];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        C[i + 3 * j] = F[0 + 3 * i] * F[0 + 3 * j] + F[1 + 3 * i] * F[1 + 3 * j] + F[2 + 3 * i] * F[2 + 3 * j];
    T trE = T(0.5) * (C[0] + C[4] + C[8] - T(3));
    for (int i = 0; i < 9; ++i) S[i] = mu * (C[i] - ((i % 4) == 0 ? T(1) : T(0)));
    S[0] += lam * trE;
    S[4] += lam * trE;
    S[8] += lam * trE;
    // F F^T (symmetric): 00 11 22 01 02 12
    FFt[0] = F[0] * F[0] + F[3] * F[3] + F[6] * F[6];
    FFt[1] = F[1] * F[1] + F[4] * F[4] + F[7] * F[7];
    FFt[2] = F[2] * F[2] + F[5] * F[5] + F[8] * F[8];
    FFt[3] = F[0] * F[1] + F[3] * F[4] + F[6] * F[7];
    FFt[4] = F[0] * F[2] + F[3] * F[5] + F[6] * F[8];
    FFt[5] = F[1] * F[2] + F[4] * F[5] + F[7] * F[8];
  }
  BT_HD void block(const T *pa, const T *pb, T *K) const {
    T fa[3], fb[3], sb[3];
    mv3(fa, F, pa);
    mv3(fb, F, pb);
    mv3(sb, S, pb);
    T d = dot3(pa, sb), m = mu * dot3(pa, pb);
    const T ff[9] = {FFt[0], FFt[3], FFt[4], FFt[3], FFt[1], FFt[5], FFt[4], FFt[5], FFt[2]};
    for (int k = 0; k < 3; ++k)
      for (int l = 0; l < 3; ++l)
        K[3 * k + l] = mu * fb[k] * fa[l] + m * ff[3 * k + l] + lam * fa[k] * fb[l] + (k == l ? d : T(0));
  }
};

// ----------------------------------------------------------------------------
// 3x3 SVD, F = U diag(S) V^T with U, V proper rotations, |S0| >= |S1| >= |S2|,
// S0, S1 >= 0 and S2 carrying the sign of det F (the convention of the
// rotation-variant SVD the reference calls through igl::svd3x3). Method
// (McAdams et al. 2011 structure): symmetric Jacobi on F^T F for V, sort the
// columns of B = F V by norm, then a Givens QR of B for U and the signed S.
// ----------------------------------------------------------------------------
template <class T>
BT_HD void jacobi_rot(T *A, T *V, int p, int q) {
  T apq = A[p + 3 * q];
  if (apq == T(0)) return;
  T theta = (A[q + 3 * q] - A[p + 3 * p]) / (T(2) * apq);
  T t = (theta >= T(0) ? T(1) : T(-1)) / (bt_abs(theta) + bt_sqrt(theta * theta + T(1)));
  T c = T(1) / bt_sqrt(t * t + T(1)), s = t * c;
  for (int k = 0; k < 3; ++k) {
    T akp = A[k + 3 * p], akq = A[k + 3 * q];
    A[k + 3 * p] = c * akp - s * akq;
    A[k + 3 * q] = s * akp + c * akq;
  }
  for (int k = 0; k < 3; ++k) {
    T apk = A[p + 3 * k], aqk = A[q + 3 * k];
    A[p + 3 * k] = c * apk - s * aqk;
    A[q + 3 * k] = s * apk + c * aqk;
  }
  for (int k = 0; k < 3; ++k) {
    T vkp = V[k + 3 * p], vkq = V[k + 3 * q];
    V[k + 3 * p] = c * vkp - s * vkq;
    V[k + 3 * q] = s * vkp + c * vkq;
  }
}

template <class T>
BT_HD void givens_rows(T *B, T *Q, int i, int k, int col) {
  T a = B[i + 3 * col], b = B[k + 3 * col];
  T r = bt_sqrt(a * a + b * b);
  T c = T(1), s = T(0);
  if (r > T(0)) {
    c = a / r;
    s = b / r;
  }
  for (int j = 0; j < 3; ++j) {
    T bi = B[i + 3 * j], bk = B[k + 3 * j];
    B[i + 3 * j] = c * bi + s * bk;
    B[k + 3 * j] = -s * bi + c * bk;
    T qi = Q[i + 3 * j], qk = Q[k + 3 * j];
    Q[i + 3 * j] = c * qi + s * qk;
    Q[k + 3 * j] = -s * qi + c * qk;
  }
}

template <class T>
BT_HD void svd3(const T *F, T *U, T *S, T *V) {
  T A[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      A[i + 3 * j] = F[0 + 3 * i] * F[0 + 3 * j] + F[1 + 3 * i] * F[1 + 3 * j] + F[2 + 3 * i] * F[2 + 3 * j];
  for (int i = 0; i < 9; ++i) V[i] = (i % 4 == 0) ? T(1) : T(0);
  if constexpr (sizeof(T) == 8) {
    // Warm start for the FP64 path (FP64 runs at a small fraction of the FP32
    // rate on this GPU): FP32 sweeps give V diagonalising F^T F to ~1e-7, two
    // Newton-Schulz steps V <- V (3 I - V^T V) / 2 in FP64 make it orthonormal
    // to rounding, and A = V^T (F^T F) V is then diagonal to ~1e-7, so the FP64
    // sweeps below (same stopping test) need one or two passes instead of ~5.
    float Af[9], Vf[9];
    for (int i = 0; i < 9; ++i) {
      Af[i] = (float)A[i];
      Vf[i] = (i % 4 == 0) ? 1.f : 0.f;
    }
    for (int s = 0; s < 6; ++s) {
      const float off = Af[3] * Af[3] + Af[6] * Af[6] + Af[7] * Af[7];
      const float dia = Af[0] * Af[0] + Af[4] * Af[4] + Af[8] * Af[8];
      if (off <= 1e-14f * dia) break;
      jacobi_rot(Af, Vf, 0, 1);
      jacobi_rot(Af, Vf, 0, 2);
      jacobi_rot(Af, Vf, 1, 2);
    }
    for (int i = 0; i < 9; ++i) V[i] = (T)Vf[i];
    for (int it = 0; it < 2; ++it) {
      T M[9], W[9], Vn[9];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
          M[i + 3 * j] = V[3 * i] * V[3 * j] + V[1 + 3 * i] * V[1 + 3 * j] + V[2 + 3 * i] * V[2 + 3 * j];
      for (int i = 0; i < 9; ++i) W[i] = ((i % 4 == 0) ? T(1.5) : T(0)) - T(0.5) * M[i];
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) Vn[i + 3 * j] = V[i] * W[3 * j] + V[i + 3] * W[1 + 3 * j] + V[i + 6] * W[2 + 3 * j];
      for (int i = 0; i < 9; ++i) V[i] = Vn[i];
    }
    T AV[9];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        AV[i + 3 * j] = A[i] * V[3 * j] + A[i + 3] * V[1 + 3 * j] + A[i + 6] * V[2 + 3 * j];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j <= i; ++j) {
        const T a = V[3 * i] * AV[3 * j] + V[1 + 3 * i] * AV[1 + 3 * j] + V[2 + 3 * i] * AV[2 + 3 * j];
        const T b = V[3 * j] * AV[3 * i] + V[1 + 3 * j] * AV[1 + 3 * i] + V[2 + 3 * j] * AV[2 + 3 * i];
        A[i + 3 * j] = A[j + 3 * i] = T(0.5) * (a + b);
      }
  }
  const int sweeps = sizeof(T) == 4 ? 6 : 12;
  for (int s = 0; s < sweeps; ++s) {
    T off = A[3] * A[3] + A[6] * A[6] + A[7] * A[7];
    T dia = A[0] * A[0] + A[4] * A[4] + A[8] * A[8];
    if (off <= (sizeof(T) == 4 ? T(1e-14) : T(1e-32)) * dia) break;
    jacobi_rot(A, V, 0, 1);
    jacobi_rot(A, V, 0, 2);
    jacobi_rot(A, V, 1, 2);
  }
  T B[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      B[i + 3 * j] = F[i + 0] * V[0 + 3 * j] + F[i + 3] * V[1 + 3 * j] + F[i + 6] * V[2 + 3 * j];
  T n[3];
  for (int j = 0; j < 3; ++j) n[j] = B[3 * j] * B[3 * j] + B[3 * j + 1] * B[3 * j + 1] + B[3 * j + 2] * B[3 * j + 2];
  // sort columns by decreasing norm
  for (int a = 0; a < 2; ++a) {
    int m = a;
    for (int b = a + 1; b < 3; ++b)
      if (n[b] > n[m]) m = b;
    if (m != a) {
      T tn = n[a];
      n[a] = n[m];
      n[m] = tn;
      for (int k = 0; k < 3; ++k) {
        T tb = B[k + 3 * a];
        B[k + 3 * a] = B[k + 3 * m];
        B[k + 3 * m] = tb;
        T tv = V[k + 3 * a];
        V[k + 3 * a] = V[k + 3 * m];
        V[k + 3 * m] = tv;
      }
    }
  }
  if (det3(V) < T(0))
    for (int k = 0; k < 3; ++k) {
      V[k + 6] = -V[k + 6];
      B[k + 6] = -B[k + 6];
    }
  T Q[9] = {T(1), T(0), T(0), T(0), T(1), T(0), T(0), T(0), T(1)};
  givens_rows(B, Q, 0, 1, 0);
  givens_rows(B, Q, 0, 2, 0);
  givens_rows(B, Q, 1, 2, 1);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) U[i + 3 * j] = Q[j + 3 * i];
  S[0] = B[0];
  S[1] = B[4];
  S[2] = B[8];
}

// Corotational, psi(S) = mu sum (s_i - 1)^2 + lambda/2 (sum s_i - 3)^2,
// pv = vol (lambda, mu) (src/psi_corotational_S.cpp:8). Hessian from the
// eigen-system of a stretch-based energy: scaling block 2 mu I + lambda 1 1^T,
// flip (dpsi_i - dpsi_j)/(s_i - s_j) = 2 mu (closed form for this law, the
// exact limit the reference approximates by perturbing F at repeated singular
// values, src/d2psi_stretch_dF2.cpp:25-28), twist (dpsi_i + dpsi_j)/(s_i + s_j).
// With frame A (alpha = A^T pa) and output frame R:
//   K_ab = R Khat R^T, Khat = 2 mu diag(alpha o beta) + lambda alpha beta^T + pair terms.
// Exact Hessian: A = V, R = U. The reference's layout (d2psi stored row-major,
// src/d2psi_stretch_dF2.cpp:37-45) equals the Hessian at F^T: A = U, R = V.
template <class T>
struct LawCorot {
  T A[9], R[9], mu2, lam, lt[3], lf[3];
  BT_HD LawCorot(const T *F, const T *pv, bool exact) {
    T U[9], S[3], V[9];
    svd3(F, U, S, V);
    for (int i = 0; i < 9; ++i) {
      A[i] = exact ? V[i] : U[i];
      R[i] = exact ? U[i] : V[i];
    }
    lam = pv[0];
    T mu = pv[1];
    mu2 = T(2) * mu;
    T tr = S[0] + S[1] + S[2] - T(3);
    T d[3];
    for (int i = 0; i < 3; ++i) d[i] = mu2 * (S[i] - T(1)) + lam * tr;
    const int P[3][2] = {{0, 1}, {0, 2}, {1, 2}};
    for (int k = 0; k < 3; ++k) {
      int i = P[k][0], j = P[k][1];
      bool repeated = bt_abs(S[i] - S[j]) < T(1e-5);
      bool stalled = !repeated && bt_abs(S[j] * S[j] - S[i] * S[i]) < T(1e-8);
      T den = S[i] + S[j];
      lf[k] = stalled ? T(0) : mu2;
      lt[k] = (stalled || den == T(0)) ? T(0) : (d[i] + d[j]) / den;
    }
  }
  BT_HD void block(const T *pa, const T *pb, T *K) const {
    T al[3], be[3];
    mtv3(al, A, pa);
    mtv3(be, A, pb);
    T H[9];
    for (int k = 0; k < 3; ++k)
      for (int l = 0; l < 3; ++l) H[3 * k + l] = lam * al[k] * be[l] + (k == l ? mu2 * al[k] * be[k] : T(0));
    const int P[3][2] = {{0, 1}, {0, 2}, {1, 2}};
    for (int k = 0; k < 3; ++k) {
      int i = P[k][0], j = P[k][1];
      T sp = T(0.5) * (lt[k] + lf[k]), sm = T(0.5) * (lf[k] - lt[k]);
      H[3 * i + i] += sp * al[j] * be[j];
      H[3 * j + j] += sp * al[i] * be[i];
      H[3 * i + j] += sm * al[j] * be[i];
      H[3 * j + i] += sm * al[i] * be[j];
    }
    // K = R H R^T (H row-major, R column-major)
    T RH[9];
    for (int k = 0; k < 3; ++k)
      for (int l = 0; l < 3; ++l)
        RH[3 * k + l] = R[k + 0] * H[0 + l] + R[k + 3] * H[3 + l] + R[k + 6] * H[6 + l];
    for (int k = 0; k < 3; ++k)
      for (int l = 0; l < 3; ++l)
        K[3 * k + l] = RH[3 * k + 0] * R[l + 0] + RH[3 * k + 1] * R[l + 3] + RH[3 * k + 2] * R[l + 6];
  }
};

// Linear elasticity, src/linear_tet_linear_elasticity_dq2.cpp:8-25 with
// src/d2psi_linear_elasticity_de2.cpp:8-24: B^T C B vol with Voigt engineering
// strains of e = sym(F) and the isotropic C; pv = vol * (lambda, mu). The
// 3x3 block of nodes a, b: lambda pa pb^T + mu pb pa^T + mu (pa . pb) I.
template <class T>
struct LawLE {
  T lam, mu;
  BT_HD LawLE(const T *, const T *pv) : lam(pv[0]), mu(pv[1]) {}
  BT_HD void block(const T *pa, const T *pb, T *K) const {
    const T ab = pa[0] * pb[0] + pa[1] * pb[1] + pa[2] * pb[2];
    for (int k = 0; k < 3; ++k)
      for (int l = 0; l < 3; ++l) K[3 * k + l] = lam * pa[k] * pb[l] + mu * pa[l] * pb[k] + (k == l ? mu * ab : T(0));
  }
};

// ARAP, src/psi_arap_S.cpp:8-11, src/dpsi_arap_dS.cpp:8-10, src/d2psi_arap_dS2.cpp:8-9:
// psi = k sum_i (s_i - 1)^2 through the same stretch machinery as the
// corotational law (src/linear_tet_arap_dq2.cpp:12-14), i.e. the corotational
// law with lambda = 0 and mu = k; params column 0 is k.
template <class T>
BT_HD void arap_pv(const T *pv, T *out) {
  out[0] = T(0);
  out[1] = pv[0];
}

#ifdef __CUDACC__
// The block law of `model` in FP64 handed to fn (a device lambda). ARAP maps
// its parameter onto the corotational law; the corotational law takes the
// reference's layout.
template <class Fn>
__device__ __forceinline__ void with_law64(int model, const double *F, const double *pv, Fn &&fn) {
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
#endif

// ----------------------------------------------------------------------------
// FP64 energy and first Piola-Kirchhoff stress (scaled by vol via pv)
// ----------------------------------------------------------------------------
// ARAP maps its parameters and continues in the corotational branch (no
// recursive call: device recursion leaves the stack size undetermined).
template <class T>
BT_HD T psi_model(int model, const T *F, const T *pv_in) {
  T pa[2];
  const T *pv = pv_in;
  if (model == MODEL_ARAP) {
    arap_pv(pv_in, pa);
    pv = pa;
    model = MODEL_COROT;
  }
  if (model == MODEL_LE) {
    // mu e:e + lambda/2 tr(e)^2, e = sym(F) (the reference's strain of q as given)
    T ee = T(0);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        const T e = T(0.5) * (F[i + 3 * j] + F[j + 3 * i]);
        ee += e * e;
      }
    const T tr = F[0] + F[4] + F[8];
    return pv[1] * ee + T(0.5) * pv[0] * tr * tr;
  }
  if (model == MODEL_NH || model == MODEL_NH_ISO) {
    T J = det3(F), I1 = T(0);
    for (int i = 0; i < 9; ++i) I1 += F[i] * F[i];
    if (model == MODEL_NH) return pv[0] * (I1 - T(3) - T(2) * bt_log(J)) + pv[1] * (J - T(1)) * (J - T(1));
    T c = bt_cbrt(J);
    return pv[0] * (I1 / (c * c) - T(3)) + pv[1] * (J - T(1)) * (J - T(1));
  }
  if (model == MODEL_STVK) {
    T C[9];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        C[i + 3 * j] = F[0 + 3 * i] * F[0 + 3 * j] + F[1 + 3 * i] * F[1 + 3 * j] + F[2 + 3 * i] * F[2 + 3 * j];
    T E[9];
    for (int i = 0; i < 9; ++i) E[i] = T(0.5) * (C[i] - ((i % 4) == 0 ? T(1) : T(0)));
    T trE = E[0] + E[4] + E[8], trEE = T(0);
    for (int i = 0; i < 9; ++i) trEE += E[i] * E[i];  // E symmetric: tr(E E) = sum E_ij^2
    return pv[1] * trEE + T(0.5) * pv[0] * trE * trE;
  }
  T U[9], S[3], V[9];
  svd3(F, U, S, V);
  T tr = S[0] + S[1] + S[2] - T(3);
  return pv[1] * ((S[0] - T(1)) * (S[0] - T(1)) + (S[1] - T(1)) * (S[1] - T(1)) + (S[2] - T(1)) * (S[2] - T(1))) +
         T(0.5) * pv[0] * tr * tr;
}

template <class T>
BT_HD void pk1_model(int model, const T *F, const T *pv_in, T *P) {
  T pa[2];
  const T *pv = pv_in;
  if (model == MODEL_ARAP) {
    arap_pv(pv_in, pa);
    pv = pa;
    model = MODEL_COROT;
  }
  if (model == MODEL_LE) {
    const T tr = F[0] + F[4] + F[8];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        P[i + 3 * j] = pv[1] * (F[i + 3 * j] + F[j + 3 * i]) + (i == j ? pv[0] * tr : T(0));
    return;
  }
  if (model == MODEL_NH || model == MODEL_NH_ISO) {
    T G[9];
    cof3(G, F);
    T J = F[0] * G[0] + F[1] * G[1] + F[2] * G[2];
    if (model == MODEL_NH) {
      T a = T(2) * pv[0], b = T(2) * pv[0] / J, c = T(2) * pv[1] * (J - T(1));
      for (int i = 0; i < 9; ++i) P[i] = a * F[i] - b * G[i] + c * G[i];
    } else {
      T I1 = T(0);
      for (int i = 0; i < 9; ++i) I1 += F[i] * F[i];
      T cr = bt_cbrt(J), Jm23 = T(1) / (cr * cr), Jm53 = Jm23 / J;
      for (int i = 0; i < 9; ++i)
        P[i] = pv[0] * (T(2) * Jm23 * F[i] - T(2) / T(3) * I1 * Jm53 * G[i]) + T(2) * pv[1] * (J - T(1)) * G[i];
    }
    return;
  }
  if (model == MODEL_STVK) {
    T C[9];
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        C[i + 3 * j] = F[0 + 3 * i] * F[0 + 3 * j] + F[1 + 3 * i] * F[1 + 3 * j] + F[2 + 3 * i] * F[2 + 3 * j];
    T trE = T(0.5) * (C[0] + C[4] + C[8] - T(3));
    T S[9];
    for (int i = 0; i < 9; ++i) S[i] = pv[1] * (C[i] - ((i % 4) == 0 ? T(1) : T(0)));
    S[0] += pv[0] * trE;
    S[4] += pv[0] * trE;
    S[8] += pv[0] * trE;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) P[i + 3 * j] = F[i] * S[3 * j] + F[i + 3] * S[3 * j + 1] + F[i + 6] * S[3 * j + 2];
    return;
  }
  // corotational with the reference's inversion fix (src/dpsi_stretch_dF.cpp:20-45)
  T U[9], S[3], V[9];
  svd3(F, U, S, V);
  T det = S[0] * S[1] * S[2];
  if (det <= T(-1e-10))
    for (int i = 0; i < 3; ++i)
      if (S[i] < T(0)) S[i] = -S[i];
  if (det3(U) <= T(0))
    for (int k = 0; k < 3; ++k) U[k + 6] = -U[k + 6];
  if (det3(V) <= T(0))
    for (int k = 0; k < 3; ++k) V[k + 6] = -V[k + 6];
  T tr = S[0] + S[1] + S[2] - T(3), d[3];
  for (int i = 0; i < 3; ++i) d[i] = T(2) * pv[1] * (S[i] - T(1)) + pv[0] * tr;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      P[i + 3 * j] = U[i] * d[0] * V[j] + U[i + 3] * d[1] * V[j + 3] + U[i + 6] * d[2] * V[j + 6];
}

// ----------------------------------------------------------------------------
// Cancellation-free energies from the displacement gradient H = F - I.
// Near the rest state psi = O(|H|^2) while the textbook forms combine O(1)
// terms (tr F^T F - 3 - 2 ln J), losing ~eps/|H|^2 relative accuracy; here
// every term is O(|H|^2) from the start.
// ----------------------------------------------------------------------------
#ifdef __CUDACC__
BT_HD double bt_log1p(double x) { return log1p(x); }
BT_HD double bt_expm1(double x) { return expm1(x); }
BT_HD float bt_log1p(float x) { return log1pf(x); }
BT_HD float bt_expm1(float x) { return expm1f(x); }
#else
BT_HD double bt_log1p(double x) { return std::log1p(x); }
BT_HD double bt_expm1(double x) { return std::expm1(x); }
BT_HD float bt_log1p(float x) { return std::log1p(x); }
BT_HD float bt_expm1(float x) { return std::expm1(x); }
#endif

// j - log1p(j) (>= 0), series sum_{k>=2} (-1)^k j^k / k for |j| < 0.02
template <class T>
BT_HD T j_minus_log1p(T j) {
  if (bt_abs(j) < T(0.02)) {
    T s = T(0);
#pragma unroll
    for (int k = 13; k >= 2; --k) s = s * j + ((k % 2 == 0) ? T(1) : T(-1)) / T(k);
    return s * j * j;
  }
  return j - bt_log1p(j);
}
// expm1(y) - y, series sum_{k>=2} y^k / k! for |y| < 0.02
template <class T>
BT_HD T expm1_minus_y(T y) {
  if (bt_abs(y) < T(0.02)) {
    T s = T(0), f = T(1);
    T c[14];
    c[0] = T(1);
#pragma unroll
    for (int k = 1; k < 14; ++k) {
      f *= T(k);
      c[k] = T(1) / f;
    }
#pragma unroll
    for (int k = 13; k >= 2; --k) s = s * y + c[k];
    return s * y * y;
  }
  return bt_expm1(y) - y;
}

// invariants of H: tr H, |H|^2, q2 = ((tr H)^2 - tr(H H))/2, det H, j = det(I + H) - 1
template <class T>
struct DispInv {
  T tr, nrm2, q2, det, j;
  BT_HD DispInv(const T *H) {
    tr = H[0] + H[4] + H[8];
    nrm2 = T(0);
    for (int i = 0; i < 9; ++i) nrm2 += H[i] * H[i];
    T trHH = T(0);
    for (int i = 0; i < 3; ++i)
      for (int k = 0; k < 3; ++k) trHH += H[i + 3 * k] * H[k + 3 * i];
    q2 = T(0.5) * (tr * tr - trHH);
    det = det3(H);
    j = tr + q2 + det;
  }
};

// psi of the displacement gradient H (F = I + H), scaled by vol via pv
template <class T>
BT_HD T psi_model_disp(int model, const T *H, const T *pv) {
  if (model == MODEL_NH || model == MODEL_NH_ISO) {
    const DispInv<T> d(H);
    const T g2 = j_minus_log1p(d.j);  // j - ln J
    if (model == MODEL_NH)
      // I1 - 3 - 2 ln J = |H|^2 + 2 (tr H - j) + 2 (j - ln J)
      return pv[0] * (d.nrm2 - T(2) * (d.q2 + d.det) + T(2) * g2) + pv[1] * d.j * d.j;
    // J^-2/3 I1 - 3 = 3 g1 + 2 g2 - 2 (q2 + det) + |H|^2 + e (2 tr H + |H|^2),
    // e = J^-2/3 - 1 = expm1(y), y = -2/3 ln J, g1 = expm1(y) - y
    const T L = bt_log1p(d.j);
    const T y = T(-2) / T(3) * L;
    const T g1 = expm1_minus_y(y);
    const T e = g1 + y;
    return pv[0] * (T(3) * g1 + T(2) * g2 - T(2) * (d.q2 + d.det) + d.nrm2 + e * (T(2) * d.tr + d.nrm2)) +
           pv[1] * d.j * d.j;
  }
  if (model == MODEL_STVK) {
    // E = (H + H^T + H^T H) / 2
    T E[9];
    for (int i = 0; i < 3; ++i)
      for (int k = 0; k < 3; ++k) {
        T hth = H[0 + 3 * i] * H[0 + 3 * k] + H[1 + 3 * i] * H[1 + 3 * k] + H[2 + 3 * i] * H[2 + 3 * k];
        E[i + 3 * k] = T(0.5) * (H[i + 3 * k] + H[k + 3 * i] + hth);
      }
    T trE = E[0] + E[4] + E[8], trEE = T(0);
    for (int i = 0; i < 9; ++i) trEE += E[i] * E[i];
    return pv[1] * trEE + T(0.5) * pv[0] * trE * trE;
  }
  T F[9];
  for (int i = 0; i < 9; ++i) F[i] = H[i] + ((i % 4) == 0 ? T(1) : T(0));
  return psi_model(model, F, pv);
}

// ----------------------------------------------------------------------------
// PSD projection helpers for one element (simple_psd_fix, src/simple_psd_fix.cpp)
// K = B^T S B with B = Phi^T (x) I3 (Phi = 4x3 stack of phi_a^T). The
// translations span null(B) and are eigenvectors of K with eigenvalue 0, so
// the projected K is  (Q (x) I) W max(L, tol) W^T (Q^T (x) I) + tol/4 (1 1^T (x) I)
// with Phi = Q R (thin QR) and M = (R (x) I) S (R^T (x) I) = W L W^T (9x9).
// Fast test: min eig M >= tol  <=>  S - tol (G^-1 (x) I) is PSD, G = Phi^T Phi.
// ----------------------------------------------------------------------------

// packed lower-triangular index of a symmetric 9x9 (i >= j)
BT_HD constexpr int p9(int i, int j) { return i >= j ? i * (i + 1) / 2 + j : j * (j + 1) / 2 + i; }

// 9x9 symmetric S from a block law, packed: S[(k + 3 i), (l + 3 j)] = block(e_i, e_j)[k][l]
template <class Law, class T>
BT_HD void law_matrix9p(const Law &law, T *S) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j <= i; ++j) {
      T ei[3] = {T(0), T(0), T(0)}, ej[3] = {T(0), T(0), T(0)};
      ei[i] = T(1);
      ej[j] = T(1);
      T K[9];
      law.block(ei, ej, K);
#pragma unroll
      for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int l = 0; l < 3; ++l)
          if ((k + 3 * i) >= (l + 3 * j)) S[p9(k + 3 * i, l + 3 * j)] = K[3 * k + l];
    }
}

// Cholesky test of a packed symmetric 9x9 (overwritten); true if all pivots > 0.
template <class T>
BT_HD bool chol9p_ok(T *A) {
  bool ok = true;
#pragma unroll
  for (int j = 0; j < 9; ++j) {
    T d = A[p9(j, j)];
#pragma unroll
    for (int k = 0; k < j; ++k) d -= A[p9(j, k)] * A[p9(j, k)];
    ok = ok && (d > T(0));
    const T s = bt_sqrt(d > T(0) ? d : T(1));
    A[p9(j, j)] = s;
    const T inv = T(1) / s;
#pragma unroll
    for (int i = j + 1; i < 9; ++i) {
      T v = A[p9(i, j)];
#pragma unroll
      for (int k = 0; k < j; ++k) v -= A[p9(i, k)] * A[p9(j, k)];
      A[p9(i, j)] = v * inv;
    }
  }
  return ok;
}

// inverse of a symmetric 3x3 (column-major)
template <class T>
BT_HD void inv3(T *R, const T *A) {
  T G[9];
  cof3(G, A);
  T J = A[0] * G[0] + A[1] * G[1] + A[2] * G[2];
  T inv = T(1) / J;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) R[i + 3 * j] = G[j + 3 * i] * inv;
}

// phi: 4 gradients (phi[a][d]). G = Phi^T Phi.
template <class T>
BT_HD void gram3(T *G, const T (*phi)[3]) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      T s = T(0);
#pragma unroll
      for (int a = 0; a < 4; ++a) s += phi[a][i] * phi[a][j];
      G[i + 3 * j] = s;
    }
}

// fast-path test on the element law: true when every non-translational
// eigenvalue of the element matrix is >= tol (nothing to project).
//
// In FP32 the test accepts eigenvalues down to tol - 1e-6 tr(M)/9: an
// eigenvalue that close to zero is within the rounding of the FP32
// eigen-decomposition the slow path would run (its absolute error is ~1e-7 of
// the largest eigenvalue), and leaving it changes the element matrix by at most
// that band (~1e-6 relative). This keeps near-rest elements, whose three
// rotation modes have numerically-zero eigenvalues, off the slow path. FP64
// (host checks) keeps the exact test.
template <class Law, class T>
BT_HD bool psd_fast_ok(const Law &law, const T (*phi)[3], T tol) {
  T S[45], G[9], Gi[9];
  law_matrix9p(law, S);
  gram3(G, phi);
  inv3(Gi, G);
  T c = tol;
  if (sizeof(T) == 4) {
    T trM = T(0);  // tr(M) = tr(S (G (x) I))
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        T tb = T(0);
#pragma unroll
        for (int k = 0; k < 3; ++k) tb += S[p9(k + 3 * i, k + 3 * j)];
        trM += G[i + 3 * j] * tb;
      }
    c = tol - T(1e-6) * bt_abs(trM) / T(9);
  }
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j <= i; ++j)
#pragma unroll
      for (int k = 0; k < 3; ++k) S[p9(k + 3 * i, k + 3 * j)] -= c * Gi[i + 3 * j];
  return chol9p_ok(S);
}

// thin QR of Phi (4x3) by modified Gram-Schmidt on its columns: Phi = Q R
template <class T>
BT_HD void qr_phi(const T (*phi)[3], T (*Q)[3], T *Rm) {
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    T v[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) v[r] = phi[r][j];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      if (i < j) {
        T d = T(0);
#pragma unroll
        for (int r = 0; r < 4; ++r) d += Q[r][i] * v[r];
        Rm[i + 3 * j] = d;
#pragma unroll
        for (int r = 0; r < 4; ++r) v[r] -= d * Q[r][i];
      } else if (i > j) {
        Rm[i + 3 * j] = T(0);
      }
    }
    T nrm = T(0);
#pragma unroll
    for (int r = 0; r < 4; ++r) nrm += v[r] * v[r];
    nrm = bt_sqrt(nrm);
    Rm[j + 3 * j] = nrm;
    const T inv = nrm > T(0) ? T(1) / nrm : T(0);
#pragma unroll
    for (int r = 0; r < 4; ++r) Q[r][j] = v[r] * inv;
  }
}

// Cyclic Jacobi on a packed symmetric 9x9 (overwritten: eigenvalues on the
// diagonal), W = eigenvectors (column-major 9x9). Rotation indices are
// compile-time so A and W stay in registers.
template <class T>
BT_HD void jacobi9p(T *A, T *W, int sweeps) {
#pragma unroll
  for (int i = 0; i < 81; ++i) W[i] = (i % 10 == 0) ? T(1) : T(0);
  for (int s = 0; s < sweeps; ++s) {
    T off = T(0), dia = T(0);
#pragma unroll
    for (int i = 0; i < 9; ++i) {
      dia += A[p9(i, i)] * A[p9(i, i)];
#pragma unroll
      for (int j = 0; j < i; ++j) off += A[p9(i, j)] * A[p9(i, j)];
    }
    if (off <= (sizeof(T) == 4 ? T(1e-14) : T(1e-32)) * dia) break;
#pragma unroll
    for (int p = 0; p < 8; ++p)
#pragma unroll
      for (int q = p + 1; q < 9; ++q) {
        const T apq = A[p9(p, q)];
        if (apq != T(0)) {
          const T theta = (A[p9(q, q)] - A[p9(p, p)]) / (T(2) * apq);
          const T t = (theta >= T(0) ? T(1) : T(-1)) / (bt_abs(theta) + bt_sqrt(theta * theta + T(1)));
          const T c = T(1) / bt_sqrt(t * t + T(1)), sn = t * c;
          A[p9(p, p)] -= t * apq;
          A[p9(q, q)] += t * apq;
          A[p9(p, q)] = T(0);
#pragma unroll
          for (int k = 0; k < 9; ++k) {
            if (k != p && k != q) {
              const T akp = A[p9(k, p)], akq = A[p9(k, q)];
              A[p9(k, p)] = c * akp - sn * akq;
              A[p9(k, q)] = sn * akp + c * akq;
            }
          }
#pragma unroll
          for (int k = 0; k < 9; ++k) {
            const T wkp = W[k + 9 * p], wkq = W[k + 9 * q];
            W[k + 9 * p] = c * wkp - sn * wkq;
            W[k + 9 * q] = sn * wkp + c * wkq;
          }
        }
      }
  }
}

// Slow path, step 1 (once per element): N = W max(L, tol) W^T (packed, 45)
// with M = (R (x) I) S (R^T (x) I) = W L W^T.
template <class Law, class T>
BT_HD_NOINLINE void psd_eig_N(const Law &law, const T (*phi)[3], T tol, T *N) {
  T M[45];
  {
    T S[45], Q[4][3], Rm[9];
    law_matrix9p(law, S);
    qr_phi(phi, Q, Rm);
    // M[(k + 3c), (l + 3d)] = sum_{i,j} R[c][i] R[d][j] S[(k + 3i), (l + 3j)]  (R upper triangular)
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int d = 0; d <= c; ++d)
#pragma unroll
        for (int k = 0; k < 3; ++k)
#pragma unroll
          for (int l = 0; l < 3; ++l) {
            if ((k + 3 * c) < (l + 3 * d)) continue;
            T acc = T(0);
#pragma unroll
            for (int i = 0; i < 3; ++i)
#pragma unroll
              for (int j = 0; j < 3; ++j)
                if (i >= c && j >= d) acc += Rm[c + 3 * i] * Rm[d + 3 * j] * S[p9(k + 3 * i, l + 3 * j)];
            M[p9(k + 3 * c, l + 3 * d)] = acc;
          }
  }
  T W[81];
  jacobi9p(M, W, sizeof(T) == 4 ? 10 : 30);
  T lam[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) lam[i] = M[p9(i, i)] < tol ? tol : M[p9(i, i)];
#pragma unroll
  for (int i = 0; i < 9; ++i)
#pragma unroll
    for (int j = 0; j <= i; ++j) {
      T acc = T(0);
#pragma unroll
      for (int k = 0; k < 9; ++k) acc += W[i + 9 * k] * lam[k] * W[j + 9 * k];
      N[p9(i, j)] = acc;
    }
}

// Slow path, step 2 (per incidence): blocks K_ab (b = 0..3) of row a from the
// projected N (packed), without the tol/4 translation term.
template <class T>
BT_HD void psd_blocks_from_N(const T *N, const T (*phi)[3], int a, T (*out)[9]) {
  T Q[4][3], Rm[9];
  qr_phi(phi, Q, Rm);
#pragma unroll
  for (int b = 0; b < 4; ++b)
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
      for (int l = 0; l < 3; ++l) {
        T acc = T(0);
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
          for (int d = 0; d < 3; ++d) acc += Q[a][c] * Q[b][d] * N[p9(k + 3 * c, l + 3 * d)];
        out[b][3 * k + l] = acc;
      }
}

// Both steps (used by host tests and by callers without a pre-pass)
template <class Law, class T>
BT_HD void psd_row_slow(const Law &law, const T (*phi)[3], T tol, int a, T (*out)[9]) {
  T N[45];
  psd_eig_N(law, phi, tol, N);
  psd_blocks_from_N(N, phi, a, out);
}

}  // namespace bartels
