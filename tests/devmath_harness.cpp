// Host build of the library's element math (bartels_gb300/csrc/devmath.cuh) so
// that CPU tests can compare the laws the CUDA kernels use with the oracle.
#include "devmath.cuh"

using namespace bartels;

template <class T>
static void block_t(int model, const T *F, const T *pv, const T *pa, const T *pb, int exact, T *K) {
  if (model == MODEL_NH) LawNH<T>(F, pv).block(pa, pb, K);
  else if (model == MODEL_NH_ISO) LawNHIso<T>(F, pv).block(pa, pb, K);
  else if (model == MODEL_STVK) LawStVK<T>(F, pv).block(pa, pb, K);
  else if (model == MODEL_LE) LawLE<T>(F, pv).block(pa, pb, K);
  else if (model == MODEL_ARAP) {
    T pc[2];
    arap_pv(pv, pc);
    LawCorot<T>(F, pc, exact != 0).block(pa, pb, K);
  } else LawCorot<T>(F, pv, exact != 0).block(pa, pb, K);
}

// 12x12 element Hessian from the block laws (row-major out[12*(3a+k) + 3b+l]),
// optionally PSD-projected the way the kernel does it.
template <class T, class Law>
static void elem_t(const Law &law, const T (*phi)[3], int psd, T tol, T *out) {
  for (int a = 0; a < 4; ++a) {
    T K[4][9];
    bool slow = psd && !psd_fast_ok(law, phi, tol);
    if (slow) psd_row_slow(law, phi, tol, a, K);
    else
      for (int b = 0; b < 4; ++b) law.block(phi[a], phi[b], K[b]);
    for (int b = 0; b < 4; ++b)
      for (int k = 0; k < 3; ++k)
        for (int l = 0; l < 3; ++l) out[12 * (3 * a + k) + 3 * b + l] = K[b][3 * k + l] + (psd ? (k == l ? tol / 4 : 0) : 0);
  }
}

template <class T>
static int element_hessian_t(int model, const T *F, const T *pv, const T *dphi9, int exact, int psd, T tol, T *out) {
  T phi[4][3];
  for (int d = 0; d < 3; ++d) {
    phi[1][d] = dphi9[d];
    phi[2][d] = dphi9[3 + d];
    phi[3][d] = dphi9[6 + d];
    phi[0][d] = -(phi[1][d] + phi[2][d] + phi[3][d]);
  }
  int slow = 0;
  auto run = [&](const auto &law) {
    slow = psd && !psd_fast_ok(law, phi, tol);
    elem_t<T>(law, phi, psd, tol, out);
  };
  if (model == MODEL_NH) run(LawNH<T>(F, pv));
  else if (model == MODEL_NH_ISO) run(LawNHIso<T>(F, pv));
  else if (model == MODEL_STVK) run(LawStVK<T>(F, pv));
  else if (model == MODEL_LE) run(LawLE<T>(F, pv));
  else if (model == MODEL_ARAP) {
    T pc[2];
    arap_pv(pv, pc);
    run(LawCorot<T>(F, pc, exact != 0));
  } else run(LawCorot<T>(F, pv, exact != 0));
  return slow;
}

extern "C" {
void dm_block_d(int model, const double *F, const double *pv, const double *pa, const double *pb, int exact,
                double *K) {
  block_t<double>(model, F, pv, pa, pb, exact, K);
}
void dm_block_f(int model, const float *F, const float *pv, const float *pa, const float *pb, int exact, float *K) {
  block_t<float>(model, F, pv, pa, pb, exact, K);
}
int dm_element_hessian_d(int model, const double *F, const double *pv, const double *dphi9, int exact, int psd,
                         double tol, double *out) {
  return element_hessian_t<double>(model, F, pv, dphi9, exact, psd, tol, out);
}
int dm_element_hessian_f(int model, const float *F, const float *pv, const float *dphi9, int exact, int psd, float tol,
                         float *out) {
  return element_hessian_t<float>(model, F, pv, dphi9, exact, psd, tol, out);
}
double dm_psi_d(int model, const double *F, const double *pv) { return psi_model<double>(model, F, pv); }
void dm_pk1_d(int model, const double *F, const double *pv, double *P) { pk1_model<double>(model, F, pv, P); }
void dm_svd3_d(const double *F, double *U, double *S, double *V) { svd3<double>(F, U, S, V); }
void dm_svd3_f(const float *F, float *U, float *S, float *V) { svd3<float>(F, U, S, V); }
void dm_def_grad_d(const double *x0, const double *x1, const double *x2, const double *x3, const double *dphi9,
                   int add_identity, double *F) {
  def_grad<double>(F, x0, x1, x2, x3, dphi9, add_identity != 0);
}
}

extern "C" double dm_psi_disp_d(int model, const double *H, const double *pv) {
  return psi_model_disp<double>(model, H, pv);
}
