// extern "C" entry points (include/bartels_gpu.h).
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "devmath.cuh"
#include "amg_internal.cuh"
#include "internal.cuh"
#include "lpcg_internal.cuh"

namespace bartels {
int plan_set_element_data(bartels_mesh_plan plan, const double *dphidX, const double *vol, const double *params,
                          const double *density);
void plan_free(bartels_mesh_plan plan);
int launch_prep_u(bartels_ctx ctx, bartels_mesh_plan plan, const double *x, const double *q_base, double scale,
                  bool displacement, float4 *u);
int launch_hess(bartels_ctx ctx, bartels_mesh_plan plan, int model, int psd_mode, const float4 *u, int add_identity,
                float cK, float cM, float tol, int flags, float *values);
int assemble_elements64(bartels_ctx ctx, bartels_mesh_plan plan, const double *Ke, double *values);
int assemble_vector64(bartels_ctx ctx, bartels_mesh_plan plan, const double *ge, double *g);
int launch_mass64(bartels_ctx ctx, bartels_mesh_plan plan, const double *density, const double *vol,
                  double *values);
int newton_iterate(bartels_ctx ctx, bartels_mesh_plan plan, const bartels_newton_params &p, double *x,
                   double g0_norm, int *done, bartels_newton_report *rep);
int newton_solve(bartels_ctx ctx, bartels_mesh_plan plan, const bartels_newton_params &p, double *x,
                 bartels_newton_report *rep);
int csr_search_direction(bartels_ctx ctx, int n, const int *rp, const int *ci, const double *vals, const double *g,
                         double *d, const bartels_pcg_params &prm, bartels_pcg_report *rep);
int advance_implicit_euler(bartels_ctx ctx, bartels_mesh_plan plan, double dt, const double *v);
int plan_spmv(bartels_ctx ctx, bartels_mesh_plan plan, const float *values, const float *x, float *y);
int plan_precond_apply(bartels_ctx ctx, bartels_mesh_plan plan, const float *values, const float *r, float *z,
                       int *levels);
int noalloc_gradient(bartels_ctx ctx, bartels_mesh_plan plan, int model, const double *q_d, double *g_d);
int plan_pcg(bartels_ctx ctx, bartels_mesh_plan plan, const float *values, const double *b, double *x,
             const bartels_pcg_params &prm, bartels_pcg_report *rep);
int plan_set_segments(bartels_mesh_plan plan, int nseg, const int *voff, const int64_t *toff);
int plan_pcg_spmv_time(bartels_ctx ctx, bartels_mesh_plan plan, const float *values, const float *x, float *y,
                       int reps, double *us);
int plan_autotune_hessian(bartels_ctx ctx, bartels_mesh_plan plan, int model, const double *q, int force,
                          int *chunk_out, int *block_out);
int plan_set_hessian_tuning(bartels_mesh_plan plan, int chunk, int block);
int newton_gradient(bartels_ctx ctx, bartels_mesh_plan plan, const bartels_newton_params &p, const double *x,
                    double *g);
int newton_energy(bartels_ctx ctx, bartels_mesh_plan plan, const bartels_newton_params &p, const double *x,
                  double *energy_host);
int plan_autotune(bartels_ctx ctx, bartels_mesh_plan plan, const float *values, int force, int *spmv_out,
                  int *tri_out);
int segment_sumsq(bartels_ctx ctx, int nseg, const int *off, const double *v, double *out);
}  // namespace bartels

using namespace bartels;

namespace {

bool valid_model(int m) { return m >= 0 && m <= 5; }

// Linear elasticity takes the reference's (Young's modulus, Poisson ratio) per
// tet (src/d2psi_linear_elasticity_de2.cpp:10-11); the kernels use the Lame
// pair (lambda, mu). Returns params itself for every other model.
const double *model_params(int model, const double *params, int nT, std::vector<double> &buf) {
  if (model != BARTELS_LINEAR_ELASTICITY || !params) return params;
  buf.resize(2 * (size_t)nT);
  for (int t = 0; t < nT; ++t) {
    const double E = params[t], nu = params[t + (size_t)nT];
    buf[t] = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
    buf[t + (size_t)nT] = E / (2.0 * (1.0 + nu));
  }
  return buf.data();
}

int check_ctx(bartels_ctx ctx) {
  if (!ctx) return fail(BARTELS_E_INVALID_ARG, "null context");
  BT_CUDA(cudaSetDevice(ctx->device));
  return BARTELS_OK;
}

int check_plan(bartels_ctx ctx, bartels_mesh_plan plan) {
  BT_CHECK(check_ctx(ctx));
  if (!plan) return fail(BARTELS_E_INVALID_ARG, "null plan");
  if (plan->ctx != ctx) return fail(BARTELS_E_INVALID_ARG, "plan belongs to another context");
  return BARTELS_OK;
}

// upload a 3nV host vector into a context staging buffer
int stage_vec(bartels_ctx ctx, DevBuf &buf, const double *h, size_t n, double **d) {
  BT_CHECK(buf.ensure(sizeof(double) * std::max<size_t>(n, 1)));
  if (n) BT_CUDA(cudaMemcpyAsync(buf.p, h, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
  *d = buf.as<double>();
  return BARTELS_OK;
}

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace

extern "C" {

const char *bartels_status_string(int s) {
  switch (s) {
    case BARTELS_OK: return "ok";
    case BARTELS_E_INVALID_ARG: return "invalid argument";
    case BARTELS_E_NONFINITE: return "non-finite value";
    case BARTELS_E_NOT_CONVERGED: return "not converged";
    case BARTELS_E_DEVICE: return "CUDA device error";
    case BARTELS_E_TIMEOUT: return "timeout";
    case BARTELS_E_UNSUPPORTED: return "unsupported input";
    case BARTELS_E_NO_DEVICE: return "no CUDA device";
    default: return "unknown status";
  }
}

const char *bartels_last_error(void) { return last_error_cstr(); }

int bartels_ctx_create(int device, bartels_ctx *out) {
  if (!out) return fail(BARTELS_E_INVALID_ARG, "null output");
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess || count == 0) return fail(BARTELS_E_NO_DEVICE, "no CUDA device available");
  if (device < 0 || device >= count) return fail(BARTELS_E_INVALID_ARG, "device index out of range");
  BT_CUDA(cudaSetDevice(device));
  auto ctx = new bartels_ctx_s;
  ctx->device = device;
  BT_CUDA(cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device));
  BT_CUDA(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
  BT_CUDA(cudaMallocHost(&ctx->host_scalars, 64 * sizeof(double)));
  if (const char *e = std::getenv("BARTELS_SPMV_LANES")) {
    const int g = std::atoi(e);
    if (g == 4 || g == 8 || g == 16) ctx->spmv_lanes = g;
  }
  if (const char *e = std::getenv("BARTELS_TRI_LANES")) {
    const int g = std::atoi(e);
    if (g == 4 || g == 8) ctx->tri_lanes = g;
  }
  *out = ctx;
  return BARTELS_OK;
}

int bartels_ctx_destroy(bartels_ctx ctx) {
  if (!ctx) return BARTELS_OK;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  ctx->partials.release();
  ctx->scalars.release();
  ctx->stage_a.release();
  ctx->stage_b.release();
  ctx->stage_c.release();
  ctx->stage_d.release();
  ctx->stage_e.release();
  if (ctx->host_scalars) cudaFreeHost(ctx->host_scalars);
  cudaStreamDestroy(ctx->stream);
  delete ctx;
  return BARTELS_OK;
}

int bartels_ctx_synchronize(bartels_ctx ctx) {
  BT_CHECK(check_ctx(ctx));
  BT_CUDA(cudaStreamSynchronize(ctx->stream));
  return BARTELS_OK;
}

void *bartels_ctx_stream(bartels_ctx ctx) { return ctx ? (void *)ctx->stream : nullptr; }
int64_t bartels_ctx_kernel_launches(bartels_ctx ctx) { return ctx ? ctx->launches : 0; }

int bartels_tetmesh_dphi_dX(bartels_ctx ctx, int nV, const double *V, int nT, const int *E, double *dphidX) {
  BT_CHECK(check_ctx(ctx));
  if (nV < 0 || nT < 0 || (!V && nV) || (!E && nT) || (!dphidX && nT))
    return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  if (nT == 0) return BARTELS_OK;
  std::vector<double> X(3 * (size_t)nV);
  for (int v = 0; v < nV; ++v)
    for (int d = 0; d < 3; ++d) X[3 * (size_t)v + d] = V[v + (size_t)nV * d];
  std::vector<int4> E4(nT);
  for (int t = 0; t < nT; ++t) {
    E4[t] = make_int4(E[t], E[t + (size_t)nT], E[t + 2 * (size_t)nT], E[t + 3 * (size_t)nT]);
    const int id[4] = {E4[t].x, E4[t].y, E4[t].z, E4[t].w};
    for (int a = 0; a < 4; ++a)
      if (id[a] < 0 || id[a] >= nV) return fail(BARTELS_E_INVALID_ARG, "element index out of range");
  }
  BT_CHECK(ctx->stage_a.ensure(sizeof(double) * X.size()));
  BT_CHECK(ctx->stage_b.ensure(sizeof(int4) * E4.size()));
  BT_CHECK(ctx->stage_c.ensure(sizeof(double) * 12 * (size_t)nT));
  BT_CUDA(cudaMemcpyAsync(ctx->stage_a.p, X.data(), sizeof(double) * X.size(), cudaMemcpyHostToDevice, ctx->stream));
  BT_CUDA(cudaMemcpyAsync(ctx->stage_b.p, E4.data(), sizeof(int4) * E4.size(), cudaMemcpyHostToDevice, ctx->stream));
  BT_CHECK(launch_dphi_vol(ctx, nV, ctx->stage_a.as<double>(), nT, ctx->stage_b.as<int4>(), ctx->stage_c.as<double>(),
                           nullptr, nullptr));
  BT_CUDA(cudaMemcpyAsync(dphidX, ctx->stage_c.p, sizeof(double) * 12 * (size_t)nT, cudaMemcpyDeviceToHost,
                          ctx->stream));
  BT_CUDA(cudaStreamSynchronize(ctx->stream));
  return BARTELS_OK;
}

int bartels_tetmesh_volume(bartels_ctx ctx, int nV, const double *V, int nT, const int *E, double *vol) {
  BT_CHECK(check_ctx(ctx));
  if (nV < 0 || nT < 0 || (!V && nV) || (!E && nT) || (!vol && nT)) return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  if (nT == 0) return BARTELS_OK;
  std::vector<double> X(3 * (size_t)nV);
  for (int v = 0; v < nV; ++v)
    for (int d = 0; d < 3; ++d) X[3 * (size_t)v + d] = V[v + (size_t)nV * d];
  std::vector<int4> E4(nT);
  for (int t = 0; t < nT; ++t) {
    E4[t] = make_int4(E[t], E[t + (size_t)nT], E[t + 2 * (size_t)nT], E[t + 3 * (size_t)nT]);
    const int id[4] = {E4[t].x, E4[t].y, E4[t].z, E4[t].w};
    for (int a = 0; a < 4; ++a)
      if (id[a] < 0 || id[a] >= nV) return fail(BARTELS_E_INVALID_ARG, "element index out of range");
  }
  BT_CHECK(ctx->stage_a.ensure(sizeof(double) * X.size()));
  BT_CHECK(ctx->stage_b.ensure(sizeof(int4) * E4.size()));
  BT_CHECK(ctx->stage_c.ensure(sizeof(double) * (size_t)nT));
  BT_CUDA(cudaMemcpyAsync(ctx->stage_a.p, X.data(), sizeof(double) * X.size(), cudaMemcpyHostToDevice, ctx->stream));
  BT_CUDA(cudaMemcpyAsync(ctx->stage_b.p, E4.data(), sizeof(int4) * E4.size(), cudaMemcpyHostToDevice, ctx->stream));
  BT_CHECK(launch_dphi_vol(ctx, nV, ctx->stage_a.as<double>(), nT, ctx->stage_b.as<int4>(), nullptr, nullptr,
                           ctx->stage_c.as<double>()));
  BT_CUDA(cudaMemcpyAsync(vol, ctx->stage_c.p, sizeof(double) * (size_t)nT, cudaMemcpyDeviceToHost, ctx->stream));
  BT_CUDA(cudaStreamSynchronize(ctx->stream));
  return BARTELS_OK;
}

int bartels_plan_create(bartels_ctx ctx, int nV, const double *V, int nT, const int *E, bartels_mesh_plan *out) {
  BT_CHECK(check_ctx(ctx));
  if (!out || nV <= 0 || nT < 0 || !V || (!E && nT)) return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  auto plan = new bartels_mesh_plan_s;
  plan->ctx = ctx;
  plan->nV = nV;
  plan->nT = nT;
  int s = plan_build(plan, V, E);
  if (s != BARTELS_OK) {
    plan_free(plan);
    delete plan;
    return s;
  }
  *out = plan;
  return BARTELS_OK;
}

int bartels_plan_destroy(bartels_mesh_plan plan) {
  if (!plan) return BARTELS_OK;
  cudaSetDevice(plan->ctx->device);
  cudaStreamSynchronize(plan->ctx->stream);
  plan_free(plan);
  delete plan;
  return BARTELS_OK;
}

int bartels_plan_set_element_data(bartels_mesh_plan plan, const double *dphidX, const double *vol,
                                  const double *params, const double *density) {
  if (!plan) return fail(BARTELS_E_INVALID_ARG, "null plan");
  BT_CHECK(check_ctx(plan->ctx));
  return plan_set_element_data(plan, dphidX, vol, params, density);
}

int bartels_plan_csr_size(bartels_mesh_plan plan, int *n, int64_t *nnz) {
  if (!plan) return fail(BARTELS_E_INVALID_ARG, "null plan");
  if (n) *n = 3 * plan->nV;
  if (nnz) *nnz = 9 * plan->nnzb;
  return BARTELS_OK;
}

int bartels_plan_csr_pattern(bartels_mesh_plan plan, int *row_ptr, int *col_idx) {
  if (!plan) return fail(BARTELS_E_INVALID_ARG, "null plan");
  BT_CHECK(check_ctx(plan->ctx));
  BT_CHECK(plan_build_csr_pattern(plan));
  bartels_ctx ctx = plan->ctx;
  if (row_ptr)
    BT_CUDA(cudaMemcpyAsync(row_ptr, plan->csr_rp, sizeof(int) * (3 * (size_t)plan->nV + 1), cudaMemcpyDeviceToHost,
                            ctx->stream));
  if (col_idx)
    BT_CUDA(cudaMemcpyAsync(col_idx, plan->csr_col, sizeof(int) * 9 * (size_t)plan->nnzb, cudaMemcpyDeviceToHost,
                            ctx->stream));
  BT_CUDA(cudaStreamSynchronize(ctx->stream));
  return BARTELS_OK;
}

int bartels_tetmesh_q(bartels_ctx ctx, bartels_mesh_plan plan, int model, const double *q, const double *dphidX,
                      const double *vol, const double *params, double *energy_out) {
  BT_CHECK(check_plan(ctx, plan));
  if (!valid_model(model) || !q || !energy_out) return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  std::vector<double> pbuf;
  BT_CHECK(plan_set_element_data(plan, dphidX, vol, model_params(model, params, plan->nT, pbuf), nullptr));
  double *dq;
  BT_CHECK(stage_vec(ctx, ctx->stage_e, q, 3 * (size_t)plan->nV, &dq));
  BT_CHECK(ctx->scalars.ensure(64 * sizeof(double)));
  ObjectiveDev obj;
  BT_CHECK(energy(ctx, plan, model, obj, dq, ctx->scalars.as<double>()));
  BT_CUDA(cudaMemcpyAsync(ctx->host_scalars, ctx->scalars.p, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  BT_CUDA(cudaStreamSynchronize(ctx->stream));
  *energy_out = ctx->host_scalars[0];
  if (!std::isfinite(*energy_out)) return fail(BARTELS_E_NONFINITE, "energy is not finite (J <= 0 for Neo-Hookean?)");
  return BARTELS_OK;
}

int bartels_tetmesh_dq(bartels_ctx ctx, bartels_mesh_plan plan, int model, const double *q, const double *dphidX,
                       const double *vol, const double *params, double *g) {
  BT_CHECK(check_plan(ctx, plan));
  if (!valid_model(model) || !q || !g) return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  std::vector<double> pbuf;
  BT_CHECK(plan_set_element_data(plan, dphidX, vol, model_params(model, params, plan->nT, pbuf), nullptr));
  const size_t n = 3 * (size_t)plan->nV;
  double *dq;
  BT_CHECK(stage_vec(ctx, ctx->stage_e, q, n, &dq));
  BT_CHECK(plan->w_vec.ensure(sizeof(double) * (3 * n + 16)));
  ObjectiveDev obj;
  BT_CHECK(gradient(ctx, plan, model, obj, dq, plan->w_vec.as<double>()));
  BT_CUDA(cudaMemcpyAsync(g, plan->w_vec.p, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
  BT_CUDA(cudaStreamSynchronize(ctx->stream));
  for (size_t i = 0; i < n; ++i)
    if (!std::isfinite(g[i])) return fail(BARTELS_E_NONFINITE, "gradient is not finite");
  return BARTELS_OK;
}

int bartels_tetmesh_dq2(bartels_ctx ctx, bartels_mesh_plan plan, int model, const double *q, const double *dphidX,
                        const double *vol, const double *params, int psd_mode, double psd_tol, int flags,
                        double *csr_values) {
  BT_CHECK(check_plan(ctx, plan));
  if (!valid_model(model) || !q || !csr_values || (psd_mode != BARTELS_PSD_NONE && psd_mode != BARTELS_PSD_SIMPLE_FIX))
    return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  std::vector<double> pbuf;
  BT_CHECK(plan_set_element_data(plan, dphidX, vol, model_params(model, params, plan->nT, pbuf), nullptr));
  const size_t n = 3 * (size_t)plan->nV;
  const int64_t nnz = 9 * plan->nnzb;
  double *dq;
  BT_CHECK(stage_vec(ctx, ctx->stage_e, q, n, &dq));
  BT_CHECK(plan->w_u.ensure(2 * sizeof(float4) * (size_t)plan->nV));
  BT_CHECK(plan->w_values.ensure(sizeof(float) * nnz));
  BT_CHECK(ctx->stage_d.ensure(sizeof(double) * nnz));
  float4 *u = plan->w_u.as<float4>();
  BT_CHECK(launch_prep_u(ctx, plan, dq, nullptr, 1.0, plan->dphi_matches_rest, u));
  BT_CHECK(launch_hess(ctx, plan, model, psd_mode, u, plan->dphi_matches_rest ? 1 : 0, 1.f, 0.f, (float)psd_tol, flags,
                       plan->w_values.as<float>()));
  BT_CHECK(values_to_double(ctx, plan->w_values.as<float>(), ctx->stage_d.as<double>(), nnz));
  BT_CUDA(cudaMemcpyAsync(csr_values, ctx->stage_d.p, sizeof(double) * nnz, cudaMemcpyDeviceToHost, ctx->stream));
  BT_CUDA(cudaStreamSynchronize(ctx->stream));
  return BARTELS_OK;
}

#define BT_NAMED(name, M)                                                                                         \
  int bartels_tetmesh_##name##_q(bartels_ctx c, bartels_mesh_plan p, const double *q, const double *d,          \
                                 const double *v, const double *pr, double *e) {                                 \
    return bartels_tetmesh_q(c, p, M, q, d, v, pr, e);                                                          \
  }                                                                                                             \
  int bartels_tetmesh_##name##_dq(bartels_ctx c, bartels_mesh_plan p, const double *q, const double *d,         \
                                  const double *v, const double *pr, double *g) {                               \
    return bartels_tetmesh_dq(c, p, M, q, d, v, pr, g);                                                         \
  }                                                                                                             \
  int bartels_tetmesh_##name##_dq2(bartels_ctx c, bartels_mesh_plan p, const double *q, const double *d,        \
                                   const double *v, const double *pr, int psd, double tol, double *vals) {      \
    return bartels_tetmesh_dq2(c, p, M, q, d, v, pr, psd, tol, 0, vals);                                        \
  }
BT_NAMED(neohookean, BARTELS_NEOHOOKEAN)
BT_NAMED(stvk, BARTELS_STVK)
BT_NAMED(corotational, BARTELS_COROTATIONAL)
BT_NAMED(arap, BARTELS_ARAP)
BT_NAMED(linear_elasticity, BARTELS_LINEAR_ELASTICITY)
#undef BT_NAMED

int bartels_tetmesh_mass_matrix(bartels_ctx ctx, bartels_mesh_plan plan, const double *density, const double *vol,
                                double *csr_values) {
  BT_CHECK(check_plan(ctx, plan));
  if (!csr_values) return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  const size_t nT = (size_t)plan->nT;
  const int64_t nnz = 9 * plan->nnzb;
  BT_CHECK(plan_set_element_data(plan, nullptr, vol, nullptr, density));
  BT_CHECK(ctx->stage_d.ensure(sizeof(double) * nnz));
  BT_CHECK(launch_mass64(ctx, plan, plan->density, plan->vol, ctx->stage_d.as<double>()));
  (void)nT;
  BT_CUDA(cudaMemcpyAsync(csr_values, ctx->stage_d.p, sizeof(double) * nnz, cudaMemcpyDeviceToHost, ctx->stream));
  BT_CUDA(cudaStreamSynchronize(ctx->stream));
  return BARTELS_OK;
}

int bartels_plan_assemble_matrix(bartels_ctx ctx, bartels_mesh_plan plan, const double *Ke, double *csr_values) {
  BT_CHECK(check_plan(ctx, plan));
  if (!Ke || !csr_values) return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  const int64_t nnz = 9 * plan->nnzb;
  double *dK;
  BT_CHECK(stage_vec(ctx, ctx->stage_e, Ke, 144 * (size_t)plan->nT, &dK));
  BT_CHECK(ctx->stage_d.ensure(sizeof(double) * nnz));
  BT_CHECK(assemble_elements64(ctx, plan, dK, ctx->stage_d.as<double>()));
  BT_CUDA(cudaMemcpyAsync(csr_values, ctx->stage_d.p, sizeof(double) * nnz, cudaMemcpyDeviceToHost, ctx->stream));
  BT_CUDA(cudaStreamSynchronize(ctx->stream));
  return BARTELS_OK;
}

int bartels_plan_assemble_vector(bartels_ctx ctx, bartels_mesh_plan plan, const double *ge, double *g) {
  BT_CHECK(check_plan(ctx, plan));
  if (!ge || !g) return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  const size_t n = 3 * (size_t)plan->nV;
  double *dge;
  BT_CHECK(stage_vec(ctx, ctx->stage_e, ge, 12 * (size_t)plan->nT, &dge));
  BT_CHECK(plan->w_vec.ensure(sizeof(double) * (n + 16)));
  BT_CHECK(assemble_vector64(ctx, plan, dge, plan->w_vec.as<double>()));
  BT_CUDA(cudaMemcpyAsync(g, plan->w_vec.p, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
  BT_CUDA(cudaStreamSynchronize(ctx->stream));
  return BARTELS_OK;
}

int bartels_tetmesh_const_ext_force(bartels_ctx ctx, bartels_mesh_plan plan, const double *vol,
                                    const double traction[3], double *f) {
  BT_CHECK(check_plan(ctx, plan));
  if (!traction || !f) return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  BT_CHECK(plan_set_element_data(plan, nullptr, vol, nullptr, nullptr));
  const size_t n = 3 * (size_t)plan->nV;
  BT_CHECK(ctx->stage_d.ensure(sizeof(double) * n));
  BT_CHECK(ext_force(ctx, plan, traction, ctx->stage_d.as<double>()));
  BT_CUDA(cudaMemcpyAsync(f, ctx->stage_d.p, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
  BT_CUDA(cudaStreamSynchronize(ctx->stream));
  return BARTELS_OK;
}

int bartels_fixed_point_constraint_matrix(int nV, int dim, const int *fixed, int nfix, int *rows, int *row_ptr,
                                          int *col_idx, double *values) {
  if (nV < 0 || dim <= 0 || nfix < 0 || (nfix && !fixed)) return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  for (int i = 1; i < nfix; ++i)
    if (fixed[i] <= fixed[i - 1]) return fail(BARTELS_E_INVALID_ARG, "fixed indices must be sorted ascending");
  for (int i = 0; i < nfix; ++i)
    if (fixed[i] < 0 || fixed[i] >= nV) return fail(BARTELS_E_INVALID_ARG, "fixed index out of range");
  const int nr = dim * (nV - nfix);
  if (rows) *rows = nr;
  if (!row_ptr) return BARTELS_OK;
  // src/fixed_point_constraint_matrix.cpp:20-34: single merge pass over vertices
  int jj = 0, r = 0;
  row_ptr[0] = 0;
  for (int ii = 0; ii < nV * dim; ii += dim) {
    if (jj < nfix && fixed[jj] == ii / dim) {
      jj += 1;
    } else {
      for (int kk = 0; kk < dim; ++kk) {
        if (col_idx) col_idx[r] = ii + kk;
        if (values) values[r] = 1.0;
        r++;
        row_ptr[r] = r;
      }
    }
  }
  return BARTELS_OK;
}

int bartels_find_min_vertices(int nV, const double *V, int dim, double tol, int *indices, int *count) {
  if (nV <= 0 || !V || dim < 0 || dim > 2 || !count) return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  double mn = V[(size_t)nV * dim];
  for (int v = 0; v < nV; ++v) mn = V[v + (size_t)nV * dim] < mn ? V[v + (size_t)nV * dim] : mn;
  int k = 0;
  for (int v = 0; v < nV; ++v)
    if (std::fabs(V[v + (size_t)nV * dim] - mn) <= tol) {
      if (indices) indices[k] = v;
      k++;
    }
  *count = k;
  return BARTELS_OK;
}

void bartels_pcg_default_params(bartels_pcg_params *p) {
  if (!p) return;
  p->rel_tol = 1e-8;
  p->max_iters = 20000;
  p->inner_rel_tol = 0.1;
  p->max_refinements = 40;
  p->restart = 0;
}

int bartels_search_direction_newton_sparse(bartels_ctx ctx, int n, const int *row_ptr, const int *col_idx,
                                           const double *values, const double *g, double *d,
                                           const bartels_pcg_params *params, bartels_pcg_report *report) {
  BT_CHECK(check_ctx(ctx));
  if (n < 0 || (n && (!row_ptr || !col_idx || !values || !g || !d))) return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  bartels_pcg_params p;
  bartels_pcg_default_params(&p);
  if (params) p = *params;
  bartels_pcg_report rep;
  std::memset(&rep, 0, sizeof(rep));
  if (n == 0) {
    if (report) *report = rep;
    return BARTELS_OK;
  }
  int s = csr_search_direction(ctx, n, row_ptr, col_idx, values, g, d, p, &rep);
  if (report) *report = rep;
  return s;
}

int bartels_linesearch_backtracking_bisection(int n, double *x, const double *d, bartels_objective_fn f, void *user,
                                              const double *g, int max_iterations, double alpha, double c, double p,
                                              int *status, double *alpha_out) {
  if (n < 0 || !x || !d || !f || !g || max_iterations < 0) return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  // src/linesearch_backtracking_bisection.cpp:17-30, with f(x) evaluated once
  std::vector<double> xt(n);
  double gd = 0.0;
  for (int i = 0; i < n; ++i) gd += g[i] * d[i];
  const double fx = f(x, n, user);
  int it = 0;
  for (;;) {
    for (int i = 0; i < n; ++i) xt[i] = x[i] + alpha * d[i];
    if (!(f(xt.data(), n, user) > fx + c * gd && it < max_iterations)) break;
    alpha *= p;
    it++;
  }
  for (int i = 0; i < n; ++i) x[i] += alpha * d[i];
  if (status) *status = (it == max_iterations) ? BARTELS_MAX_ITERATIONS_REACHED : BARTELS_CONVERGED;
  if (alpha_out) *alpha_out = alpha;
  return BARTELS_OK;
}

void bartels_newton_default_params(bartels_newton_params *p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->model = BARTELS_NEOHOOKEAN;
  p->psd_mode = BARTELS_PSD_NONE;
  p->psd_tol = 1e-6;
  p->dq2_flags = 0;
  p->mass_coeff = 0.0;
  p->scale = 1.0;
  p->force_scale = 1.0;
  p->gradient_tol = 1e-3;  // include/optimization_gradient_based.h:51-56
  p->relative = 0;
  p->max_iterations = 100;
  p->max_iterations_ls = 100;
  p->ls_alpha = 1.0;
  p->ls_c = 1e-8;
  p->ls_p = 0.5;
  bartels_pcg_default_params(&p->pcg);
}

int bartels_newton_set_problem(bartels_mesh_plan plan, const double *q_base, const double *x_hat, const double *f_ext,
                               const unsigned char *pinned) {
  if (!plan) return fail(BARTELS_E_INVALID_ARG, "null plan");
  bartels_ctx ctx = plan->ctx;
  BT_CHECK(check_ctx(ctx));
  const size_t n = 3 * (size_t)plan->nV;
  auto put = [&](double **dst, const double *src) -> int {
    if (!src) {
      if (*dst) cudaFree(*dst);
      *dst = nullptr;
      return BARTELS_OK;
    }
    if (!*dst) BT_CUDA(cudaMalloc(dst, sizeof(double) * n));
    BT_CUDA(cudaMemcpyAsync(*dst, src, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
    return BARTELS_OK;
  };
  BT_CHECK(put(&plan->q_base, q_base));
  BT_CHECK(put(&plan->x_hat, x_hat));
  BT_CHECK(put(&plan->f_ext, f_ext));
  // the pinned set's generation moves only when the set itself changes (the
  // multigrid hierarchy of a plan is built for one set)
  if (pinned) {
    if (plan->h_pinned.size() != (size_t)plan->nV ||
        std::memcmp(plan->h_pinned.data(), pinned, (size_t)plan->nV) != 0) {
      plan->h_pinned.assign(pinned, pinned + plan->nV);
      plan->pinned_gen++;
    }
  } else if (!plan->h_pinned.empty()) {
    plan->h_pinned.clear();
    plan->pinned_gen++;
  }
  if (pinned) {
    if (!plan->pinned) BT_CUDA(cudaMalloc(&plan->pinned, (size_t)plan->nV));
    BT_CUDA(cudaMemcpyAsync(plan->pinned, pinned, (size_t)plan->nV, cudaMemcpyHostToDevice, ctx->stream));
  } else if (plan->pinned) {
    cudaFree(plan->pinned);
    plan->pinned = nullptr;
  }
  BT_CUDA(cudaStreamSynchronize(ctx->stream));
  return BARTELS_OK;
}

int bartels_newton_solve_d(bartels_ctx ctx, bartels_mesh_plan plan, const bartels_newton_params *params, double *x_d,
                           bartels_newton_report *report) {
  BT_CHECK(check_plan(ctx, plan));
  if (!params || !x_d || !valid_model(params->model)) return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  bartels_newton_report rep;
  std::memset(&rep, 0, sizeof(rep));
  int s = newton_solve(ctx, plan, *params, x_d, &rep);
  if (report) *report = rep;
  return s;
}

int bartels_newton_solve(bartels_ctx ctx, bartels_mesh_plan plan, const bartels_newton_params *params, double *x,
                         bartels_newton_report *report) {
  BT_CHECK(check_plan(ctx, plan));
  if (!params || !x || !valid_model(params->model)) return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  const double t0 = now_s();
  const size_t n = 3 * (size_t)plan->nV;
  double *dx;
  BT_CHECK(stage_vec(ctx, ctx->stage_e, x, n, &dx));
  bartels_newton_report rep;
  std::memset(&rep, 0, sizeof(rep));
  int s = newton_solve(ctx, plan, *params, dx, &rep);
  BT_CUDA(cudaMemcpyAsync(x, dx, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
  BT_CUDA(cudaStreamSynchronize(ctx->stream));
  rep.seconds = now_s() - t0;
  if (report) *report = rep;
  return s;
}

int bartels_newton_iterate_d(bartels_ctx ctx, bartels_mesh_plan plan, const bartels_newton_params *params,
                             double *x_d, double g0_norm, int *done, bartels_newton_report *report) {
  BT_CHECK(check_plan(ctx, plan));
  if (!params || !x_d || !done || !report || !valid_model(params->model))
    return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  return newton_iterate(ctx, plan, *params, x_d, g0_norm, done, report);
}

int bartels_plan_hessian_d(bartels_ctx ctx, bartels_mesh_plan plan, int model, int psd_mode, double psd_tol,
                           int flags, double coeff_K, double coeff_M, const double *q_d, float *values_d) {
  BT_CHECK(check_plan(ctx, plan));
  if (!valid_model(model) || !q_d || (psd_mode != BARTELS_PSD_NONE && psd_mode != BARTELS_PSD_SIMPLE_FIX))
    return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  BT_CHECK(plan->w_u.ensure(2 * sizeof(float4) * (size_t)plan->nV));
  BT_CHECK(plan->w_values.ensure(sizeof(float) * 9 * (size_t)plan->nnzb));
  float4 *u = plan->w_u.as<float4>();
  BT_CHECK(launch_prep_u(ctx, plan, q_d, nullptr, 1.0, plan->dphi_matches_rest, u));
  return launch_hess(ctx, plan, model, psd_mode, u, plan->dphi_matches_rest ? 1 : 0, (float)coeff_K, (float)coeff_M,
                     (float)psd_tol, flags, values_d ? values_d : plan->w_values.as<float>());
}

int bartels_plan_spmv_d(bartels_ctx ctx, bartels_mesh_plan plan, const float *values_d, const float *x_d, float *y_d) {
  BT_CHECK(check_plan(ctx, plan));
  if (!x_d || !y_d) return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  if (!values_d) {
    if (plan->w_values.bytes < sizeof(float) * 9 * (size_t)plan->nnzb)
      return fail(BARTELS_E_INVALID_ARG, "the plan has no assembled Hessian yet");
    values_d = plan->w_values.as<float>();
  }
  return plan_spmv(ctx, plan, values_d, x_d, y_d);
}

int bartels_newton_advance_implicit_euler_d(bartels_ctx ctx, bartels_mesh_plan plan, double dt, const double *v_d) {
  BT_CHECK(check_plan(ctx, plan));
  if (!v_d) return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  return advance_implicit_euler(ctx, plan, dt, v_d);
}

int bartels_tetmesh_q_d(bartels_ctx ctx, bartels_mesh_plan plan, int model, const double *q_d, double *energy_d) {
  BT_CHECK(check_plan(ctx, plan));
  if (!valid_model(model) || !q_d || !energy_d) return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  ObjectiveDev obj;
  return energy(ctx, plan, model, obj, q_d, energy_d);
}

int bartels_tetmesh_q_elements_d(bartels_ctx ctx, bartels_mesh_plan plan, int model, const double *q_d,
                                 double *e_d) {
  BT_CHECK(check_plan(ctx, plan));
  if (!valid_model(model) || !q_d || !e_d) return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  return energy_elements(ctx, plan, model, q_d, e_d);
}

int bartels_tetmesh_dq_d(bartels_ctx ctx, bartels_mesh_plan plan, int model, const double *q_d, double *g_d) {
  BT_CHECK(check_plan(ctx, plan));
  if (!valid_model(model) || !q_d || !g_d) return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  ObjectiveDev obj;
  return gradient(ctx, plan, model, obj, q_d, g_d);
}

int bartels_tetmesh_dq_noalloc_d(bartels_ctx ctx, bartels_mesh_plan plan, int model, const double *q_d,
                                 double *g_d) {
  BT_CHECK(check_plan(ctx, plan));
  if (!valid_model(model) || !q_d || !g_d) return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  return noalloc_gradient(ctx, plan, model, q_d, g_d);
}


int bartels_lpcg_create(bartels_ctx ctx, bartels_lpcg *out) {
  BT_CHECK(check_ctx(ctx));
  if (!out) return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  return lpcg_create(ctx, out);
}

int bartels_lpcg_destroy(bartels_lpcg net) {
  if (!net) return BARTELS_OK;
  BT_CHECK(check_ctx(lpcg_ctx(net)));
  lpcg_destroy(net);
  return BARTELS_OK;
}

int bartels_lpcg_num_params(void) { return lpcg_num_params(); }

int bartels_lpcg_set_params(bartels_lpcg net, const float *params) {
  if (!net || !params) return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  BT_CHECK(check_ctx(lpcg_ctx(net)));
  return lpcg_set_params(net, params);
}

int bartels_lpcg_get_params(bartels_lpcg net, float *params, float *grad) {
  if (!net) return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  BT_CHECK(check_ctx(lpcg_ctx(net)));
  return lpcg_get_params(net, params, grad);
}

int bartels_lpcg_train_step(bartels_lpcg net, bartels_mesh_plan plan, const float *values_d,
                            const double *residual_d, int nprobes, unsigned seed, float lr, float clip,
                            double *loss) {
  if (!net || !values_d || !loss || nprobes < 0 || nprobes > 64) return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  BT_CHECK(check_plan(lpcg_ctx(net), plan));
  return lpcg_train_step(net, plan, values_d, residual_d, nprobes, seed, lr, clip, loss);
}

int bartels_lpcg_outputs(bartels_lpcg net, bartels_mesh_plan plan, const float *values_d, float *raw,
                         float *g_lower) {
  if (!net || !values_d) return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  BT_CHECK(check_plan(lpcg_ctx(net), plan));
  return lpcg_outputs(net, plan, values_d, raw, g_lower);
}

int bartels_plan_factor_size(bartels_mesh_plan plan, int64_t *nnzl_blocks, int64_t *nnzu_blocks) {
  if (!plan) return fail(BARTELS_E_INVALID_ARG, "null plan");
  BT_CHECK(check_ctx(plan->ctx));
  FactorPattern *fp;
  BT_CHECK(plan_factor_pattern(plan, &fp));
  if (nnzl_blocks) *nnzl_blocks = fp->nnzl;
  if (nnzu_blocks) *nnzu_blocks = fp->nnzu;
  return BARTELS_OK;
}

int bartels_plan_set_preconditioner(bartels_mesh_plan plan, int kind, bartels_lpcg net) {
  if (!plan) return fail(BARTELS_E_INVALID_ARG, "null plan");
  if (kind == BARTELS_PRECOND_BLOCK_JACOBI) {
    plan->precond = kind;
    plan->lpcg_net = nullptr;
    return BARTELS_OK;
  }
  if (kind == BARTELS_PRECOND_MULTIGRID) {
    plan->precond = kind;
    plan->lpcg_net = nullptr;
    return BARTELS_OK;
  }
  if ((kind != BARTELS_PRECOND_LEARNED && kind != BARTELS_PRECOND_LEARNED_MULTIGRID) || !net)
    return fail(BARTELS_E_INVALID_ARG, "unknown preconditioner");
  if (lpcg_ctx(net) != plan->ctx) return fail(BARTELS_E_INVALID_ARG, "network belongs to another context");
  plan->precond = kind;
  plan->lpcg_net = net;
  return BARTELS_OK;
}

int bartels_plan_pcg_d(bartels_ctx ctx, bartels_mesh_plan plan, const float *values_d, const double *b_d,
                       double *x_d, const bartels_pcg_params *params, bartels_pcg_report *report) {
  BT_CHECK(check_plan(ctx, plan));
  if (!b_d || !x_d || !report) return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  if (!values_d) {
    if (plan->w_values.bytes < sizeof(float) * 9 * (size_t)plan->nnzb)
      return fail(BARTELS_E_INVALID_ARG, "the plan has no assembled Hessian yet");
    values_d = plan->w_values.as<float>();
  }
  bartels_pcg_params p;
  if (params) p = *params;
  else bartels_pcg_default_params(&p);
  return plan_pcg(ctx, plan, values_d, b_d, x_d, p, report);
}

int bartels_plan_precond_apply_d(bartels_ctx ctx, bartels_mesh_plan plan, const float *values_d, const float *r_d,
                                 float *z_d, int *levels) {
  BT_CHECK(check_plan(ctx, plan));
  if (!values_d || !r_d || !z_d) return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  return plan_precond_apply(ctx, plan, values_d, r_d, z_d, levels);
}

int bartels_newton_gradient_d(bartels_ctx ctx, bartels_mesh_plan plan, const bartels_newton_params *params,
                              const double *x_d, double *g_d) {
  BT_CHECK(check_plan(ctx, plan));
  if (!params || !x_d || !g_d || !valid_model(params->model)) return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  return newton_gradient(ctx, plan, *params, x_d, g_d);
}

int bartels_newton_get_problem(bartels_mesh_plan plan, double *q_base, double *x_hat) {
  if (!plan) return fail(BARTELS_E_INVALID_ARG, "null plan");
  BT_CHECK(check_ctx(plan->ctx));
  const size_t n = 3 * (size_t)plan->nV;
  BT_CUDA(cudaStreamSynchronize(plan->ctx->stream));
  auto get = [&](double *dst, const double *src) -> int {
    if (!dst) return BARTELS_OK;
    if (!src) {
      std::memset(dst, 0, sizeof(double) * n);
      return BARTELS_OK;
    }
    BT_CUDA(cudaMemcpy(dst, src, sizeof(double) * n, cudaMemcpyDeviceToHost));
    return BARTELS_OK;
  };
  BT_CHECK(get(q_base, plan->q_base));
  return get(x_hat, plan->x_hat);
}

int bartels_newton_energy_d(bartels_ctx ctx, bartels_mesh_plan plan, const bartels_newton_params *params,
                            const double *x_d, double *energy) {
  BT_CHECK(check_plan(ctx, plan));
  if (!params || !x_d || !energy || !valid_model(params->model)) return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  return newton_energy(ctx, plan, *params, x_d, energy);
}

int bartels_plan_mg_info(bartels_mesh_plan plan, int max_levels, int *levels, int *nodes, int64_t *blocks,
                         int *coarsest) {
  if (!plan || !plan->mg) return fail(BARTELS_E_INVALID_ARG, "the plan has no multigrid hierarchy");
  const MgHierarchy *mg = plan->mg;
  const int L = (int)mg->lv.size();
  if (levels) *levels = L;
  for (int l = 0; l < L && l < max_levels; ++l) {
    if (nodes) nodes[l] = mg->lv[l].n;
    if (blocks) blocks[l] = mg->lv[l].nnzb;
  }
  if (coarsest) *coarsest = mg->dense ? 0 : (mg->coarse_blockdiag ? 1 : 2);
  return BARTELS_OK;
}

int bartels_plan_autotune(bartels_ctx ctx, bartels_mesh_plan plan, const float *values_d, int force,
                          int *spmv_lanes, int *factor_lanes) {
  BT_CHECK(check_plan(ctx, plan));
  if (!values_d) {
    if (plan->w_values.bytes < sizeof(float) * 9 * (size_t)plan->nnzb)
      return fail(BARTELS_E_INVALID_ARG, "the plan has no assembled Hessian yet");
    values_d = plan->w_values.as<float>();
  }
  return plan_autotune(ctx, plan, values_d, force, spmv_lanes, factor_lanes);
}

int bartels_plan_pcg_spmv_time_d(bartels_ctx ctx, bartels_mesh_plan plan, const float *values_d, const float *x_d,
                                 float *y_d, int reps, double *us_per_launch) {
  BT_CHECK(check_plan(ctx, plan));
  if (!x_d || !y_d || !us_per_launch || reps < 1) return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  if (!values_d) {
    if (plan->w_values.bytes < sizeof(float) * 9 * (size_t)plan->nnzb)
      return fail(BARTELS_E_INVALID_ARG, "the plan has no assembled Hessian yet");
    values_d = plan->w_values.as<float>();
  }
  return plan_pcg_spmv_time(ctx, plan, values_d, x_d, y_d, reps, us_per_launch);
}

int bartels_plan_autotune_hessian(bartels_ctx ctx, bartels_mesh_plan plan, int model, const double *q_d, int force,
                                  int *chunk_vertices, int *psd_block) {
  BT_CHECK(check_plan(ctx, plan));
  if (!q_d || !valid_model(model)) return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  return plan_autotune_hessian(ctx, plan, model, q_d, force, chunk_vertices, psd_block);
}

int bartels_plan_set_hessian_tuning(bartels_mesh_plan plan, int chunk_vertices, int psd_block) {
  if (!plan) return fail(BARTELS_E_INVALID_ARG, "null plan");
  return plan_set_hessian_tuning(plan, chunk_vertices, psd_block);
}

int bartels_plan_set_segments(bartels_mesh_plan plan, int nseg, const int *vertex_offsets,
                              const int64_t *tet_offsets) {
  if (!plan) return fail(BARTELS_E_INVALID_ARG, "null plan");
  BT_CHECK(check_ctx(plan->ctx));
  return plan_set_segments(plan, nseg, vertex_offsets, tet_offsets);
}

int bartels_plan_set_segment_active(bartels_mesh_plan plan, const unsigned char *active) {
  if (!plan || !active) return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  if (!plan->seg) return fail(BARTELS_E_INVALID_ARG, "the plan has no segments");
  plan->seg->active.assign(active, active + plan->seg->nseg);
  return BARTELS_OK;
}

int bartels_plan_segment_pcg_iterations(bartels_mesh_plan plan, int *iterations) {
  if (!plan || !iterations) return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  if (!plan->seg) return fail(BARTELS_E_INVALID_ARG, "the plan has no segments");
  for (int q = 0; q < plan->seg->nseg; ++q)
    iterations[q] = q < (int)plan->seg->last_iters.size() ? plan->seg->last_iters[q] : 0;
  return BARTELS_OK;
}

int bartels_segment_sumsq_d(bartels_ctx ctx, int nseg, const int *vertex_offsets_d, const double *v_d, double *out_d) {
  BT_CHECK(check_ctx(ctx));
  if (nseg < 0 || (nseg > 0 && (!vertex_offsets_d || !v_d || !out_d)))
    return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  return segment_sumsq(ctx, nseg, vertex_offsets_d, v_d, out_d);
}

static int gemm_entry(bartels_ctx ctx, int M, int N, int K, const void *x_d, int ldx, const void *w_d,
                      const float *bias_d, int relu, float *y_d, int ldy, int probe_polls);

int bartels_gemm_bf16_d(bartels_ctx ctx, int M, int N, int K, const void *x_d, int ldx, const void *w_d,
                        const float *bias_d, int relu, float *y_d, int ldy) {
  return gemm_entry(ctx, M, N, K, x_d, ldx, w_d, bias_d, relu, y_d, ldy, 0);
}

int bartels_gemm_bf16_wait_probe_d(bartels_ctx ctx, int M, int N, int K, const void *x_d, int ldx,
                                   const void *w_d, float *y_d, int ldy, int polls) {
  return gemm_entry(ctx, M, N, K, x_d, ldx, w_d, nullptr, 0, y_d, ldy, polls > 0 ? polls : 1);
}

static int gemm_entry(bartels_ctx ctx, int M, int N, int K, const void *x_d, int ldx, const void *w_d,
                      const float *bias_d, int relu, float *y_d, int ldy, int probe_polls) {
  BT_CHECK(check_ctx(ctx));
  if (M < 0 || !x_d || !w_d || !y_d) return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  BT_CHECK(ctx->stage_e.ensure(sizeof(int)));
  int *err = ctx->stage_e.as<int>();
  BT_CUDA(cudaMemsetAsync(err, 0, sizeof(int), ctx->stream));
  GemmArgs g;
  g.M = M;
  g.N = N;
  g.K = K;
  g.x = static_cast<const __nv_bfloat16 *>(x_d);
  g.ldx = ldx;
  g.w = static_cast<const __nv_bfloat16 *>(w_d);
  g.bias = bias_d;
  g.relu = relu;
  g.y = y_d;
  g.ldy = ldy;
  g.err = err;
  g.probe_polls = probe_polls;
  BT_CHECK(gemm_bf16(ctx, g));
  int h = 0;
  BT_CUDA(cudaMemcpyAsync(&h, err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  BT_CUDA(cudaStreamSynchronize(ctx->stream));
  if (h) return fail(BARTELS_E_TIMEOUT, "tensor-core GEMM: a bounded wait gave up");
  return BARTELS_OK;
}

}  // extern "C"
