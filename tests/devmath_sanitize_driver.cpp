// Drives the library's element math (bartels_gb300/csrc/devmath.cuh, through
// tests/devmath_harness.cpp) on the host over many deformation gradients:
// near rest, stretched, compressed, rotated, nearly degenerate and with
// repeated singular values, for every law, in FP64 and FP32, with and without
// the PSD projection. Built with -fsanitize=address,undefined by the test
// suite, so an out-of-bounds access or undefined arithmetic (signed overflow,
// bad shifts, misaligned loads) aborts the run; non-finite results where F is
// invertible fail it. Prints "devmath sanitize ok" and returns 0.
#include <cmath>
#include <cstdio>

extern "C" {
int dm_element_hessian_d(int model, const double *F, const double *pv, const double *dphi9, int exact, int psd,
                         double tol, double *out);
int dm_element_hessian_f(int model, const float *F, const float *pv, const float *dphi9, int exact, int psd,
                         float tol, float *out);
double dm_psi_d(int model, const double *F, const double *pv);
void dm_pk1_d(int model, const double *F, const double *pv, double *P);
void dm_svd3_d(const double *F, double *U, double *S, double *V);
void dm_svd3_f(const float *F, float *U, float *S, float *V);
}

#define REQUIRE(c)                                                          \
  do {                                                                      \
    if (!(c)) {                                                             \
      std::fprintf(stderr, "check failed: %s (line %d)\n", #c, __LINE__); \
      return 1;                                                             \
    }                                                                       \
  } while (0)

int main() {
  unsigned seed = 11;
  auto rnd = [&] {
    seed = seed * 1664525u + 1013904223u;
    return ((seed >> 8) & 0xFFFFF) / 1048576.0 - 0.5;
  };
  const double dphi9[9] = {1.0, 0.1, -0.2, 0.05, 1.1, 0.0, -0.1, 0.2, 0.9};
  float dphi9f[9];
  for (int i = 0; i < 9; ++i) dphi9f[i] = (float)dphi9[i];
  int cases = 0;
  for (int kind = 0; kind < 6; ++kind)
    for (int rep = 0; rep < 40; ++rep) {
      double F[9];
      for (int i = 0; i < 9; ++i) F[i] = (i % 4 == 0 ? 1.0 : 0.0);
      const double amp = kind == 0 ? 1e-7 : (kind == 1 ? 0.2 : (kind == 2 ? 0.45 : 0.05));
      for (int i = 0; i < 9; ++i) F[i] += amp * rnd();
      if (kind == 3) F[8] *= 0.3;                             // strong compression
      if (kind == 4) F[0] = F[4] = F[8] = 1.0 + 1e-9 * rnd();  // repeated singular values
      if (kind == 5) {                                         // rotation about z times a stretch
        const double a = 6.28 * rnd(), c = std::cos(a), s = std::sin(a);
        const double R[9] = {c, s, 0, -s, c, 0, 0, 0, 1};
        for (int i = 0; i < 9; ++i) F[i] = R[i] * (i % 4 == 0 ? 1.0 + 0.1 * rnd() : 1.0);
      }
      float Ff[9];
      for (int i = 0; i < 9; ++i) Ff[i] = (float)F[i];
      double U[9], S[3], V[9];
      dm_svd3_d(F, U, S, V);
      float Uf[9], Sf[3], Vf[9];
      dm_svd3_f(Ff, Uf, Sf, Vf);
      for (int model = 0; model <= 5; ++model) {
        const double pv[2] = {3e4, 1e5};
        const float pvf[2] = {3e4f, 1e5f};
        const double e = dm_psi_d(model, F, pv);
        double P[9];
        dm_pk1_d(model, F, pv, P);
        const double J = F[0] * (F[4] * F[8] - F[5] * F[7]) - F[3] * (F[1] * F[8] - F[2] * F[7]) +
                         F[6] * (F[1] * F[5] - F[2] * F[4]);
        if (J > 0.05) {
          REQUIRE(std::isfinite(e));
          for (double p : P) REQUIRE(std::isfinite(p));
        }
        for (int exact = 0; exact < 2; ++exact)
          for (int psd = 0; psd < 2; ++psd) {
            double K[144];
            float Kf[144];
            dm_element_hessian_d(model, F, pv, dphi9, exact, psd, 1e-6, K);
            dm_element_hessian_f(model, Ff, pvf, dphi9f, exact, psd, 1e-6f, Kf);
            if (J > 0.05)
              for (int i = 0; i < 144; ++i) REQUIRE(std::isfinite(K[i]) && std::isfinite(Kf[i]));
            ++cases;
          }
      }
    }
  std::printf("devmath sanitize ok (%d element Hessians)\n", cases);
  return 0;
}
