// Context, device buffers and mesh plans.
//
// A plan turns (V, E) into the structures every hot kernel reads:
//   * per-vertex incidence lists (tet id * 4 + local slot) in ascending tet
//     order, so per-vertex sums run in the element order the reference uses;
//   * the 3x3 block pattern (one block per vertex pair sharing a tet) with
//     values kept in scalar-CSR order;
//   * for every incidence the positions of the tet's four vertices inside the
//     row of the incident vertex (the element-to-CSR scatter map, 4 x 8 bit);
//   * chunks of consecutive vertices whose CSR values fit in shared memory.
// The pattern equals the one Eigen's setFromTriplets builds in src/assemble.cpp:94.
#include <omp.h>

#include <algorithm>
#include <cstring>
#include <mutex>

#include "devmath.cuh"
#include "amg_internal.cuh"
#include "internal.cuh"
#include "lpcg_internal.cuh"

namespace bartels {

static thread_local std::string g_last_error;

void set_error(const std::string &msg) { g_last_error = msg; }
int fail(int status, const std::string &msg) {
  g_last_error = msg;
  return status;
}
const char *last_error_cstr() { return g_last_error.c_str(); }

int DevBuf::ensure(size_t n) {
  if (n <= bytes) return BARTELS_OK;
  const size_t want = std::max(n, bytes + bytes / 2);
  if (p) cudaFree(p);
  p = nullptr;
  bytes = 0;
  cudaError_t e = cudaMalloc(&p, want);
  if (e != cudaSuccess) {
    p = nullptr;
    return fail(BARTELS_E_DEVICE, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  }
  bytes = want;
  return BARTELS_OK;
}

void DevBuf::release() {
  if (p) cudaFree(p);
  p = nullptr;
  bytes = 0;
}

int launch_import_dphi(bartels_ctx ctx, bartels_mesh_plan plan, const double *src_d, double *err_d);

template <class T>
static int upload(bartels_ctx ctx, T **dst, const T *src, size_t n) {
  BT_CUDA(cudaMalloc(dst, sizeof(T) * std::max<size_t>(n, 1)));
  if (n) BT_CUDA(cudaMemcpyAsync(*dst, src, sizeof(T) * n, cudaMemcpyHostToDevice, ctx->stream));
  return BARTELS_OK;
}

int plan_build(bartels_mesh_plan plan, const double *V, const int *E) {
  bartels_ctx ctx = plan->ctx;
  const int nV = plan->nV, nT = plan->nT;
  // incidences pack 4 t + a into an int (and count 4 nT of them)
  if ((int64_t)nT >= (1 << 29)) return fail(BARTELS_E_UNSUPPORTED, "more than 2^29 tets");
  // --- validate and convert layouts
  std::vector<double> X(3 * (size_t)nV);
  for (int v = 0; v < nV; ++v)
    for (int d = 0; d < 3; ++d) X[3 * (size_t)v + d] = V[v + (size_t)nV * d];
  std::vector<int4> E4(nT);
  for (int t = 0; t < nT; ++t) {
    int id[4];
    for (int a = 0; a < 4; ++a) {
      id[a] = E[t + (size_t)nT * a];
      if (id[a] < 0 || id[a] >= nV) return fail(BARTELS_E_INVALID_ARG, "element index out of range");
    }
    for (int a = 0; a < 4; ++a)
      for (int b = a + 1; b < 4; ++b)
        if (id[a] == id[b]) return fail(BARTELS_E_INVALID_ARG, "tet with a repeated vertex");
    E4[t] = make_int4(id[0], id[1], id[2], id[3]);
  }
  // --- incidence lists in tet order (counting sort by vertex, stable in t)
  std::vector<int> inc_ptr(nV + 1, 0);
  for (int t = 0; t < nT; ++t) {
    inc_ptr[E4[t].x + 1]++;
    inc_ptr[E4[t].y + 1]++;
    inc_ptr[E4[t].z + 1]++;
    inc_ptr[E4[t].w + 1]++;
  }
  for (int v = 0; v < nV; ++v) inc_ptr[v + 1] += inc_ptr[v];
  std::vector<int> inc_tet(4 * (size_t)nT);
  {
    std::vector<int> fill(inc_ptr.begin(), inc_ptr.end() - 1);
    for (int t = 0; t < nT; ++t) {
      const int id[4] = {E4[t].x, E4[t].y, E4[t].z, E4[t].w};
      for (int a = 0; a < 4; ++a) inc_tet[fill[id[a]]++] = 4 * t + a;
    }
  }
  // --- block pattern: sorted unique neighbours (self included) per vertex
  std::vector<int> nbcount(nV);
  std::vector<std::vector<int>> rows(nV);
  int bad = 0;
#pragma omp parallel for schedule(dynamic, 1024) reduction(+ : bad)
  for (int v = 0; v < nV; ++v) {
    std::vector<int> &r = rows[v];
    r.reserve(4 * (inc_ptr[v + 1] - inc_ptr[v]) + 1);
    r.push_back(v);
    for (int k = inc_ptr[v]; k < inc_ptr[v + 1]; ++k) {
      const int4 e = E4[inc_tet[k] >> 2];
      r.push_back(e.x);
      r.push_back(e.y);
      r.push_back(e.z);
      r.push_back(e.w);
    }
    std::sort(r.begin(), r.end());
    r.erase(std::unique(r.begin(), r.end()), r.end());
    nbcount[v] = (int)r.size();
    if (r.size() > 255) bad++;
  }
  if (bad) return fail(BARTELS_E_UNSUPPORTED, "a vertex has more than 254 neighbours");
  std::vector<int> brp(nV + 1, 0);
  for (int v = 0; v < nV; ++v) brp[v + 1] = brp[v] + nbcount[v];
  const int64_t nnzb = brp[nV];
  if (9 * nnzb > (int64_t)INT32_MAX) return fail(BARTELS_E_UNSUPPORTED, "more than 2^31 CSR entries");
  std::vector<int> bcol(nnzb), diag(nV);
  std::vector<uint32_t> inc_pos(4 * (size_t)nT);
  int max_nb = 0;
#pragma omp parallel for schedule(dynamic, 1024) reduction(max : max_nb)
  for (int v = 0; v < nV; ++v) {
    const std::vector<int> &r = rows[v];
    std::copy(r.begin(), r.end(), bcol.begin() + brp[v]);
    diag[v] = (int)(std::lower_bound(r.begin(), r.end(), v) - r.begin());
    max_nb = std::max(max_nb, (int)r.size());
    for (int k = inc_ptr[v]; k < inc_ptr[v + 1]; ++k) {
      const int4 e = E4[inc_tet[k] >> 2];
      const int id[4] = {e.x, e.y, e.z, e.w};
      uint32_t pos = 0;
      for (int b = 0; b < 4; ++b) {
        uint32_t j = (uint32_t)(std::lower_bound(r.begin(), r.end(), id[b]) - r.begin());
        pos |= j << (8 * b);
      }
      inc_pos[k] = pos;
    }
  }
  rows.clear();
  rows.shrink_to_fit();
  // --- chunks of consecutive vertices for the shared-memory assembly
  std::vector<int> chunks{0};
  {
    int start = 0;
    int64_t floats = 0;
    for (int v = 0; v < nV; ++v) {
      const int64_t need = 9ll * nbcount[v];
      if (need > kChunkFloats) return fail(BARTELS_E_UNSUPPORTED, "vertex row too long for shared memory");
      if (v - start >= kChunkMaxVerts || floats + need > kChunkFloats) {
        chunks.push_back(v);
        start = v;
        floats = 0;
      }
      floats += need;
    }
    if (chunks.back() != nV) chunks.push_back(nV);
  }
  plan->nnzb = nnzb;
  plan->max_row_blocks = max_nb;
  plan->nchunks = (int)chunks.size() - 1;
  plan->h_brp = brp;
  plan->h_bcol = bcol;
  plan->h_chunk_v = chunks;
  // --- upload
  BT_CHECK(upload(ctx, &plan->X, X.data(), X.size()));
  BT_CHECK(upload(ctx, &plan->E, E4.data(), E4.size()));
  BT_CHECK(upload(ctx, &plan->inc_ptr, inc_ptr.data(), inc_ptr.size()));
  BT_CHECK(upload(ctx, &plan->inc_tet, inc_tet.data(), inc_tet.size()));
  BT_CHECK(upload(ctx, &plan->inc_pos, inc_pos.data(), inc_pos.size()));
  BT_CHECK(upload(ctx, &plan->brp, brp.data(), brp.size()));
  BT_CHECK(upload(ctx, &plan->bcol, bcol.data(), bcol.size()));
  BT_CHECK(upload(ctx, &plan->diag_pos, diag.data(), diag.size()));
  BT_CHECK(upload(ctx, &plan->chunk_v, chunks.data(), chunks.size()));
  // --- element data defaults: geometry from V, params and density zero
  BT_CUDA(cudaMalloc(&plan->dphi64, sizeof(double) * 9 * std::max<size_t>(nT, 1)));
  BT_CUDA(cudaMalloc(&plan->vol, sizeof(double) * std::max<size_t>(nT, 1)));
  BT_CUDA(cudaMalloc(&plan->params, sizeof(double) * 2 * std::max<size_t>(nT, 1)));
  BT_CUDA(cudaMalloc(&plan->density, sizeof(double) * std::max<size_t>(nT, 1)));
  BT_CUDA(cudaMemsetAsync(plan->params, 0, sizeof(double) * 2 * (size_t)nT, ctx->stream));
  BT_CUDA(cudaMemsetAsync(plan->density, 0, sizeof(double) * (size_t)nT, ctx->stream));
  BT_CUDA(cudaMalloc(&plan->rec32, sizeof(TetRec32) * std::max<size_t>(nT, 1)));
  BT_CUDA(cudaMalloc(&plan->rec64, sizeof(TetRec64) * std::max<size_t>(nT, 1)));
  if (nT > 0) {
    BT_CHECK(launch_dphi_vol(ctx, nV, plan->X, nT, plan->E, nullptr, plan->dphi64, plan->vol));
    BT_CHECK(plan_refresh_records(plan));
  }
  plan->dphi_matches_rest = true;
  BT_CUDA(cudaStreamSynchronize(ctx->stream));
  return BARTELS_OK;
}

// Upload caller element data (reference layouts) into the plan.
int plan_set_element_data(bartels_mesh_plan plan, const double *dphidX, const double *vol, const double *params,
                          const double *density) {
  bartels_ctx ctx = plan->ctx;
  const size_t nT = (size_t)plan->nT;
  if (nT == 0) return BARTELS_OK;
  bool changed = false;
  if (dphidX) {
    BT_CHECK(ctx->stage_a.ensure(sizeof(double) * 12 * nT));
    BT_CHECK(ctx->stage_b.ensure(sizeof(double) * 2));
    BT_CUDA(cudaMemcpyAsync(ctx->stage_a.p, dphidX, sizeof(double) * 12 * nT, cudaMemcpyHostToDevice, ctx->stream));
    BT_CHECK(launch_import_dphi(ctx, plan, ctx->stage_a.as<double>(), ctx->stage_b.as<double>()));
    double err[2];
    BT_CUDA(cudaMemcpyAsync(err, ctx->stage_b.p, sizeof(err), cudaMemcpyDeviceToHost, ctx->stream));
    BT_CUDA(cudaStreamSynchronize(ctx->stream));
    if (!(err[0] <= 1e-9))
      return fail(BARTELS_E_UNSUPPORTED,
                  "dphidX row 0 must equal minus the sum of rows 1..3 (as linear_tetmesh_dphi_dX produces)");
    plan->dphi_matches_rest = err[1] <= 1e-6;
    changed = true;
  }
  if (vol) {
    BT_CUDA(cudaMemcpyAsync(plan->vol, vol, sizeof(double) * nT, cudaMemcpyHostToDevice, ctx->stream));
    changed = true;
  }
  if (params) {
    // column-major nT x 2 -> per-tet pairs
    std::vector<double> p(2 * nT);
    for (size_t t = 0; t < nT; ++t) {
      p[2 * t] = params[t];
      p[2 * t + 1] = params[t + nT];
    }
    BT_CUDA(cudaMemcpyAsync(plan->params, p.data(), sizeof(double) * 2 * nT, cudaMemcpyHostToDevice, ctx->stream));
    BT_CUDA(cudaStreamSynchronize(ctx->stream));
    changed = true;
  }
  if (density) {
    BT_CUDA(cudaMemcpyAsync(plan->density, density, sizeof(double) * nT, cudaMemcpyHostToDevice, ctx->stream));
    changed = true;
  }
  if (changed) BT_CHECK(plan_refresh_records(plan));
  BT_CUDA(cudaStreamSynchronize(ctx->stream));
  return BARTELS_OK;
}

void FactorPattern::release() {
  int *ptrs[] = {lrp, urp, low2up, up2low, rev};
  for (int *p : ptrs)
    if (p) cudaFree(p);
  if (meta) cudaFree(meta);
  meta = nullptr;
  lrp = urp = low2up = up2low = rev = nullptr;
  built = false;
}

// Lower / upper storage maps of a triangular factor on the plan's block
// pattern (rows are sorted, so the lower part of a row is a prefix of it).
// Chunks of at most 64 consecutive vertices whose values fit in 32 KB: the
// assembly's smaller CTA shape (more CTAs per SM, less shared memory each).
int plan_chunks64(bartels_mesh_plan plan) {
  if (plan->chunk_v64) return BARTELS_OK;
  constexpr int kVerts = 64, kFloats = kChunkFloats / 2;
  std::vector<int> chunks{0};
  int start = 0;
  int64_t floats = 0;
  for (int v = 0; v < plan->nV; ++v) {
    const int64_t need = 9ll * (plan->h_brp[v + 1] - plan->h_brp[v]);
    if (need > kFloats) return fail(BARTELS_E_UNSUPPORTED, "vertex row too long for the half-size chunks");
    if (v - start >= kVerts || floats + need > kFloats) {
      chunks.push_back(v);
      start = v;
      floats = 0;
    }
    floats += need;
  }
  if (chunks.back() != plan->nV) chunks.push_back(plan->nV);
  BT_CUDA(cudaMalloc(&plan->chunk_v64, sizeof(int) * chunks.size()));
  BT_CUDA(cudaMemcpy(plan->chunk_v64, chunks.data(), sizeof(int) * chunks.size(), cudaMemcpyHostToDevice));
  plan->nchunks64 = (int)chunks.size() - 1;
  return BARTELS_OK;
}

int plan_factor_pattern(bartels_mesh_plan plan, FactorPattern **out) {
  if (!plan->factor) plan->factor = new FactorPattern();
  FactorPattern &f = *plan->factor;
  *out = plan->factor;
  if (f.built) return BARTELS_OK;
  const int nV = plan->nV;
  const std::vector<int> &brp = plan->h_brp, &bcol = plan->h_bcol;
  std::vector<int> diag(nV), lrp(nV + 1, 0), urp(nV + 1, 0);
  for (int v = 0; v < nV; ++v) {
    const int *r = bcol.data() + brp[v];
    const int nb = brp[v + 1] - brp[v];
    diag[v] = (int)(std::lower_bound(r, r + nb, v) - r);
    lrp[v + 1] = lrp[v] + diag[v] + 1;
    urp[v + 1] = urp[v] + nb - diag[v];
  }
  const int64_t nnzl = lrp[nV], nnzu = urp[nV];
  std::vector<int> low2up(nnzl), up2low(nnzu), rev(plan->nnzb);
#pragma omp parallel for schedule(dynamic, 1024)
  for (int v = 0; v < nV; ++v) {
    const int nb = brp[v + 1] - brp[v];
    for (int b = 0; b < nb; ++b) {
      const int j = bcol[brp[v] + b];
      const int *rj = bcol.data() + brp[j];
      const int nbj = brp[j + 1] - brp[j];
      const int pos = (int)(std::lower_bound(rj, rj + nbj, v) - rj);  // v in row j
      rev[brp[v] + b] = brp[j] + pos;
      if (b <= diag[v]) {
        // lower block (v, j), j <= v  ->  upper block (j, v) of row j
        low2up[lrp[v] + b] = urp[j] + (pos - diag[j]);
      } else {
        // upper block (v, j), j > v   ->  lower block (j, v) of row j
        up2low[urp[v] + (b - diag[v])] = lrp[j] + pos;
      }
    }
    up2low[urp[v]] = lrp[v] + diag[v];  // diagonal block
  }
  std::vector<int4> meta(nV);
  int64_t lseg = 0, useg = 0;
  for (int v = 0; v < nV; ++v) {
    const int nb = brp[v + 1] - brp[v];
    meta[v] = make_int4(brp[v], (int)lseg, (int)useg, diag[v] | (nb << 16));
    lseg += 3ll * padded_row(diag[v] + 1);
    useg += 3ll * padded_row(nb - diag[v]);
  }
  if (lseg > INT32_MAX || useg > INT32_MAX) return fail(BARTELS_E_UNSUPPORTED, "factor storage above 2^31 entries");
  f.lsize = lseg;
  f.usize = useg;
  bartels_ctx ctx = plan->ctx;
  BT_CHECK(upload(ctx, &f.meta, meta.data(), meta.size()));
  BT_CHECK(upload(ctx, &f.lrp, lrp.data(), lrp.size()));
  BT_CHECK(upload(ctx, &f.urp, urp.data(), urp.size()));
  BT_CHECK(upload(ctx, &f.low2up, low2up.data(), low2up.size()));
  BT_CHECK(upload(ctx, &f.up2low, up2low.data(), up2low.size()));
  BT_CHECK(upload(ctx, &f.rev, rev.data(), rev.size()));
  BT_CUDA(cudaStreamSynchronize(ctx->stream));
  f.nnzl = nnzl;
  f.nnzu = nnzu;
  f.built = true;
  return BARTELS_OK;
}

void lpcg_plan_release(bartels_mesh_plan plan);

void plan_free(bartels_mesh_plan plan) {
  if (plan->factor) {
    plan->factor->release();
    delete plan->factor;
    plan->factor = nullptr;
  }
  lpcg_plan_release(plan);
  mg_destroy(plan->mg);
  plan->mg = nullptr;
  delete plan->seg;
  plan->seg = nullptr;
  if (plan->chunk_v64) cudaFree(plan->chunk_v64);
  if (plan->pad_off) cudaFree(plan->pad_off);
  plan->chunk_v64 = nullptr;
  void *ptrs[] = {plan->X,        plan->E,      plan->dphi64,  plan->vol,     plan->params,  plan->density,
                  plan->rec32,    plan->rec64,  plan->inc_ptr, plan->inc_tet, plan->inc_pos, plan->brp,
                  plan->bcol,     plan->diag_pos, plan->chunk_v, plan->csr_rp, plan->csr_col, plan->q_base,
                  plan->x_hat,    plan->f_ext,  plan->pinned};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  plan->w_values.release();
  plan->w_minv.release();
  plan->w_vec.release();
  plan->w_grad_e.release();
  plan->w_energy.release();
  plan->w_u.release();
  plan->w_pcg.release();
  plan->w_psd.release();
  plan->w_spmv.release();
  plan->w_vpad.release();
}

}  // namespace bartels
