// Internal declarations of the GB300 tet-mesh library: context and plan
// structures, per-tet records, error plumbing and small device math.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <string>
#include <utility>
#include <vector>

#include "bartels_gpu.h"

namespace bartels {

// ----------------------------------------------------------------- errors ---
void set_error(const std::string &msg);
int fail(int status, const std::string &msg);
const char *last_error_cstr();

#define BT_CUDA(call)                                                                       \
  do {                                                                                      \
    cudaError_t e_ = (call);                                                                \
    if (e_ != cudaSuccess)                                                                  \
      return ::bartels::fail(BARTELS_E_DEVICE, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

#define BT_CHECK(call)            \
  do {                            \
    int s_ = (call);              \
    if (s_ != BARTELS_OK) return s_; \
  } while (0)

// Launch bookkeeping: every kernel launch goes through this so the context can
// count launches and report launch errors.
#define BT_LAUNCH(ctx, kernel, grid, block, smem, ...)                                     \
  do {                                                                                      \
    kernel<<<(grid), (block), (smem), (ctx)->stream>>>(__VA_ARGS__);                        \
    (ctx)->launches++;                                                                      \
    cudaError_t e_ = cudaGetLastError();                                                    \
    if (e_ != cudaSuccess)                                                                  \
      return ::bartels::fail(BARTELS_E_DEVICE, std::string("launch ") + #kernel + ": " + cudaGetErrorString(e_)); \
  } while (0)

// The same with programmatic dependent launch (the kernel must call pdl_wait()
// before it reads anything its predecessor writes).
#define BT_LAUNCH_PDL(ctx, kernel, grid, block, smem, ...)                                 \
  do {                                                                                      \
    cudaLaunchConfig_t cfg_ = {};                                                           \
    cfg_.gridDim = dim3(grid);                                                              \
    cfg_.blockDim = dim3(block);                                                            \
    cfg_.dynamicSmemBytes = (smem);                                                         \
    cfg_.stream = (ctx)->stream;                                                            \
    cudaLaunchAttribute at_[1];                                                             \
    at_[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;                         \
    at_[0].val.programmaticStreamSerializationAllowed = 1;                                  \
    cfg_.attrs = at_;                                                                       \
    cfg_.numAttrs = 1;                                                                      \
    cudaError_t e_ = cudaLaunchKernelEx(&cfg_, kernel, __VA_ARGS__);                         \
    (ctx)->launches++;                                                                      \
    if (e_ != cudaSuccess)                                                                  \
      return ::bartels::fail(BARTELS_E_DEVICE, std::string("launch ") + #kernel + ": " + cudaGetErrorString(e_)); \
  } while (0)

// ------------------------------------------------------------------ records ---
// FP32 record of one tet for the Hessian kernels: 64 bytes, one aligned line
// pair, loaded with four 16-byte loads.
//   idx     : the 4 vertex ids
//   dphi    : gradients of shape functions 1..3 (rows 1..3 of the reference's
//             4x3 dphidX), phi_0 = -(phi_1 + phi_2 + phi_3)
//   pv      : vol * params (both laws are linear in params)
//   mass    : density * vol
struct alignas(16) TetRec32 {
  int4 idx;
  float dphi[9];  // dphi[3*(a-1) + d] = d phi_a / d X_d, a = 1..3
  float pv[2];
  float mass;
};
static_assert(sizeof(TetRec32) == 64, "TetRec32 must be 64 bytes");

// FP64 record for energy / gradient kernels (thread per tet): 128 bytes.
struct alignas(16) TetRec64 {
  double dphi[9];
  double pv[2];
  double mass;
  int4 idx;
  double vol;
  double pad;
};
static_assert(sizeof(TetRec64) == 128, "TetRec64 must be 128 bytes");

struct FactorPattern;  // lower / upper block storage maps (learned preconditioner)
struct LpcgPlanState;  // per-plan buffers of the learned preconditioner
struct MgHierarchy;    // aggregation multigrid hierarchy of a plan

// Packed meshes: the plan's vertices and tets as independent segments
// (instances), each with its own PCG scalars and line-search step.
struct SegInfo {
  int nseg = 0;
  int *voff = nullptr;           // nseg + 1 vertex offsets (device)
  int64_t *toff = nullptr;       // nseg + 1 tet offsets (device)
  int *vseg = nullptr;           // segment of each vertex (device)
  int *tseg = nullptr;           // segment of each tet (device)
  std::vector<int> h_voff;
  std::vector<int64_t> h_toff;
  std::vector<unsigned char> active;  // segments still solved (host)
  // per-segment PCG scalars and line-search buffers (device)
  double *rz = nullptr, *rr = nullptr, *tol2 = nullptr, *abs2 = nullptr, *red = nullptr, *red2 = nullptr;
  float *alpha = nullptr, *beta = nullptr;
  int *done = nullptr, *iters = nullptr;
  double *alpha64 = nullptr;     // line-search steps
  double *et = nullptr, *ev = nullptr;  // per-tet and per-vertex energy-difference terms
  std::vector<int> last_iters;   // PCG iterations per segment of the last solve (host)
  std::vector<void *> allocs;
  ~SegInfo();
};

// Device buffer with geometric growth.
struct DevBuf {
  void *p = nullptr;
  size_t bytes = 0;
  int ensure(size_t n);
  void release();
  template <class T>
  T *as() const { return static_cast<T *>(p); }
};

}  // namespace bartels

struct bartels_ctx_s {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  int64_t launches = 0;
  // lanes per vertex row in the block-layout SpMV (4, 8 or 16; tuned per GPU,
  // overridable with BARTELS_SPMV_LANES)
  int spmv_lanes = 8;
  // lanes per vertex row in the triangular factor passes (4 or 8; BARTELS_TRI_LANES)
  int tri_lanes = 4;
  // autotuner results per size bucket (floor(log2 nV)): {SpMV lanes, factor-pass lanes}
  std::map<int, std::pair<int, int>> tune_cache;
  // Hessian autotuner results per size bucket: {vertices per assembly CTA, PSD block size}
  std::map<int, std::pair<int, int>> tune_cache_hess;
  // pinned host staging for small read-backs
  double *host_scalars = nullptr;
  // device scratch for reductions
  bartels::DevBuf partials, scalars;
  // large host<->device staging (grown on demand)
  bartels::DevBuf stage_a, stage_b, stage_c, stage_d, stage_e;
};

struct bartels_mesh_plan_s {
  bartels_ctx ctx = nullptr;
  int nV = 0, nT = 0;
  // rest geometry
  double *X = nullptr;        // 3 nV interleaved rest positions
  int4 *E = nullptr;          // nT
  // element data (FP64 master copies)
  double *dphi64 = nullptr;   // nT x 9 (rows 1..3 of dphidX, per tet contiguous)
  double *vol = nullptr;      // nT
  double *params = nullptr;   // nT x 2 (per tet contiguous)
  double *density = nullptr;  // nT
  bartels::TetRec32 *rec32 = nullptr;
  bartels::TetRec64 *rec64 = nullptr;
  // incidence lists: for vertex v, entries inc_ptr[v] .. inc_ptr[v+1]-1 in tet order
  int *inc_ptr = nullptr;     // nV + 1
  int *inc_tet = nullptr;     // 4 nT : tet * 4 + local slot
  uint32_t *inc_pos = nullptr;// 4 nT : 4 x 8-bit block positions in the row of v
  // block pattern (3x3 blocks), values stored in scalar-CSR order
  int *brp = nullptr;         // nV + 1
  int *bcol = nullptr;        // nnzb
  int *diag_pos = nullptr;    // nV: position of the diagonal block within its row
  int64_t nnzb = 0;
  int max_row_blocks = 0;
  // assembly chunks (consecutive vertex ranges whose values fit in shared memory)
  int *chunk_v = nullptr;     // nchunks + 1
  int nchunks = 0;
  // half-size chunks (<= 64 vertices, 32 KB), made when the tuning asks for them
  int *chunk_v64 = nullptr;
  // padded copy of the FP32 values for the PCG loop's SpMV: vertex v's three
  // scalar rows start at pad_off[v] (pad_total entries in all), each padded
  // with zeros to a multiple of 4 entries; w_vpad holds the copy
  int *pad_off = nullptr;
  int64_t pad_total = 0;
  int nchunks64 = 0;
  // Hessian tuning: vertices per assembly CTA (128, or 64 with chunk_v64) and
  // threads per CTA of the PSD pre-pass kernels (64, 128 or 256)
  int hess_chunk = 128, psd_block = 128;
  std::vector<int> h_brp, h_bcol, h_chunk_v;  // host copies
  // lazily built scalar CSR pattern (device)
  int *csr_rp = nullptr, *csr_col = nullptr;
  // Newton problem data
  double *q_base = nullptr, *x_hat = nullptr, *f_ext = nullptr;
  unsigned char *pinned = nullptr;
  int pinned_gen = 0;  // incremented whenever the pinned set changes
  std::vector<unsigned char> h_pinned;  // host copy of the pinned set (empty: none)
  // true when dphidX is the rest shape's own (F = I + sum (u_a - u_0) phi_a^T)
  bool dphi_matches_rest = true;
  // triangular-factor pattern and learned-preconditioner buffers (built on first use)
  bartels::FactorPattern *factor = nullptr;
  bartels::LpcgPlanState *lpcg = nullptr;
  int precond = BARTELS_PRECOND_BLOCK_JACOBI;
  // lanes per vertex row chosen by the autotuner for this plan (0: the context's)
  int spmv_lanes = 0, tri_lanes = 0;
  bartels_lpcg lpcg_net = nullptr;
  // aggregation multigrid hierarchy (built on first use for the current pinned set)
  bartels::MgHierarchy *mg = nullptr;
  // packed-mesh segments (nullptr: one system)
  bartels::SegInfo *seg = nullptr;
  // solver workspace
  bartels::DevBuf w_values, w_minv, w_vec, w_grad_e, w_energy, w_u, w_pcg, w_psd, w_spmv, w_vpad;
};

namespace bartels {

constexpr int kChunkFloats = 16384;  // 64 KB of shared memory per assembly CTA
constexpr int kChunkMaxVerts = 128;


// Kernel-side entry points implemented in the .cu files.
int plan_build(bartels_mesh_plan plan, const double *V_host, const int *E_host);
// the half-size assembly chunks (built once, on first use)
int plan_chunks64(bartels_mesh_plan plan);
int plan_refresh_records(bartels_mesh_plan plan);
int plan_build_csr_pattern(bartels_mesh_plan plan);

int launch_dphi_vol(bartels_ctx ctx, int nV, const double *X3, int nT, const int4 *E, double *dphidX_colmajor,
                    double *dphi9, double *vol);

struct ObjectiveDev {
  double mass_coeff = 0.0;  // multiplies the mass terms
  double scale = 1.0;       // q = q_base + scale * x
  double force_scale = 0.0; // multiplies x^T f_ext
  const double *q_base = nullptr;
  const double *x_hat = nullptr;
  const double *f_ext = nullptr;
  const unsigned char *pinned = nullptr;
};

// energy of the objective at x; result (FP64) left in *d_out (device) and
// returned through the pinned scalar if host_out != nullptr.
int energy(bartels_ctx ctx, bartels_mesh_plan plan, int model, const ObjectiveDev &obj, const double *x,
           double *d_out);
// per-tet (et, nT) and per-vertex force (ev, nV) terms of f(x + alpha_s d) - f(x)
// with each tet / vertex taking its segment's step alpha_seg[s] (0: term 0)
int energy_diff_seg(bartels_ctx ctx, bartels_mesh_plan plan, int model, const ObjectiveDev &obj, const double *x,
                    const double *dx, const double *alpha_seg, const int *tseg, const int *vseg, double *et,
                    double *ev);
// energy of every tet (nT doubles) at positions q
int energy_elements(bartels_ctx ctx, bartels_mesh_plan plan, int model, const double *q, double *e);
int gradient(bartels_ctx ctx, bartels_mesh_plan plan, int model, const ObjectiveDev &obj, const double *x,
             double *g);
// f(x + alpha dx) - f(x), element by element (line search)
int energy_diff(bartels_ctx ctx, bartels_mesh_plan plan, int model, const ObjectiveDev &obj, const double *x,
                const double *dx, double alpha, double *d_out);
int mass_values(bartels_ctx ctx, bartels_mesh_plan plan, float *values32, double *values64);
int ext_force(bartels_ctx ctx, bartels_mesh_plan plan, const double traction[3], double *f);
int values_to_double(bartels_ctx ctx, const float *v32, double *v64, int64_t n);

// sums n doubles deterministically into *out (device)
int reduce_sum(bartels_ctx ctx, const double *in, int n, double *out);
int dot(bartels_ctx ctx, const double *a, const double *b, int n, double *out);

}  // namespace bartels
