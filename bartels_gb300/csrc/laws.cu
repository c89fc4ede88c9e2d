// Pointwise material laws over a batch of deformation gradients: the
// reference's psi_<law>_F, dpsi_<law>_dF and d2psi_<law>_dF2
// (src/psi_neohookean_F.cpp:31, src/dpsi_neohookean_dF.cpp:58-66,
// src/d2psi_neohookean_dF2.cpp:185-283, src/psi_stvk_F.cpp:11-12,
// src/dpsi_stvk_dF.cpp:25-33, src/d2psi_stvk_dF2.cpp:26-106, and the stretch
// family src/psi_stretch_F.cpp, src/dpsi_stretch_dF.cpp,
// src/d2psi_stretch_dF2.cpp behind the corotational and ARAP laws), as the
// MATLAB gateways matlab/dpsi_neohookean_dF.cpp, matlab/d2psi_neohookean_dF2.cpp
// and matlab/d2psi_stvk_dF2.cpp apply them element by element.
//
// One thread per deformation gradient, FP64, with the same device laws as the
// mesh kernels: psi_model, pk1_model, and d2psi/dF2 read off the Hessian block
// laws, d2psi/dF(k,i)dF(l,j) = block(e_i, e_j)[k][l].
#include "devmath.cuh"
#include "internal.cuh"

#include <algorithm>
#include <vector>

namespace bartels {
namespace {

__global__ void k_laws(int model, int n, const double *F, const double *pv, double *psi, double *dpsi,
                       double *d2psi) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  double f[9], p[2];
  for (int r = 0; r < 9; ++r) f[r] = F[t + (size_t)n * r];
  p[0] = pv[t];
  p[1] = pv[t + (size_t)n];
  if (psi) psi[t] = psi_model(model, f, p);
  if (dpsi) {
    double P[9];
    pk1_model(model, f, p, P);
    for (int r = 0; r < 9; ++r) dpsi[t + (size_t)n * r] = P[r];
  }
  if (d2psi) {
    double *H = d2psi + 81 * (size_t)t;
    with_law64(model, f, p, [&](const auto &law) {
      for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
          double ei[3] = {0.0, 0.0, 0.0}, ej[3] = {0.0, 0.0, 0.0}, K[9];
          ei[i] = 1.0;
          ej[j] = 1.0;
          law.block(ei, ej, K);
          for (int k = 0; k < 3; ++k)
            for (int l = 0; l < 3; ++l) H[(k + 3 * i) + 9 * (l + 3 * j)] = K[3 * k + l];
        }
    });
  }
}

}  // namespace
}  // namespace bartels

using namespace bartels;

extern "C" int bartels_pointwise_laws(bartels_ctx ctx, int model, int n, const double *F, const double *params,
                                      double *psi, double *dpsi, double *d2psi) {
  if (!ctx) return fail(BARTELS_E_INVALID_ARG, "null context");
  if (model < 0 || model > 5 || n < 0 || (n > 0 && (!F || !params)))
    return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  if ((size_t)n > ((size_t)1 << 31) / 81) return fail(BARTELS_E_UNSUPPORTED, "too many deformation gradients");
  if (n == 0) return BARTELS_OK;
  BT_CUDA(cudaSetDevice(ctx->device));
  const size_t N = (size_t)n;
  // linear elasticity: (Young's modulus, Poisson ratio) -> (lambda, mu) as at the mesh entry points
  std::vector<double> pb(params, params + 2 * N);
  if (model == BARTELS_LINEAR_ELASTICITY)
    for (size_t t = 0; t < N; ++t) {
      const double E = params[t], nu = params[t + N];
      pb[t] = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
      pb[t + N] = E / (2.0 * (1.0 + nu));
    }
  BT_CHECK(ctx->stage_a.ensure(sizeof(double) * 11 * N));
  const size_t out = (psi ? N : 0) + (dpsi ? 9 * N : 0) + (d2psi ? 81 * N : 0);
  BT_CHECK(ctx->stage_b.ensure(sizeof(double) * std::max<size_t>(out, 1)));
  double *dF = ctx->stage_a.as<double>(), *dp = dF + 9 * N;
  double *o = ctx->stage_b.as<double>();
  double *o_psi = psi ? o : nullptr;
  double *o_dpsi = dpsi ? o + (psi ? N : 0) : nullptr;
  double *o_d2 = d2psi ? o + (psi ? N : 0) + (dpsi ? 9 * N : 0) : nullptr;
  BT_CUDA(cudaMemcpyAsync(dF, F, sizeof(double) * 9 * N, cudaMemcpyHostToDevice, ctx->stream));
  BT_CUDA(cudaMemcpyAsync(dp, pb.data(), sizeof(double) * 2 * N, cudaMemcpyHostToDevice, ctx->stream));
  BT_LAUNCH(ctx, k_laws, (unsigned)((N + 127) / 128), 128, 0, model, n, dF, dp, o_psi, o_dpsi, o_d2);
  if (psi) BT_CUDA(cudaMemcpyAsync(psi, o_psi, sizeof(double) * N, cudaMemcpyDeviceToHost, ctx->stream));
  if (dpsi) BT_CUDA(cudaMemcpyAsync(dpsi, o_dpsi, sizeof(double) * 9 * N, cudaMemcpyDeviceToHost, ctx->stream));
  if (d2psi) BT_CUDA(cudaMemcpyAsync(d2psi, o_d2, sizeof(double) * 81 * N, cudaMemcpyDeviceToHost, ctx->stream));
  BT_CUDA(cudaStreamSynchronize(ctx->stream));  // pb lives on this stack frame
  return BARTELS_OK;
}
