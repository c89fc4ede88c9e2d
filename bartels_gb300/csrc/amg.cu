// Aggregation multigrid preconditioner for the Newton systems.
//
// No counterpart in the reference, whose search direction factors the Hessian
// with Eigen::SparseLU (src/search_direction_newton_sparse.cpp:12-18). Block-
// Jacobi PCG needs O(1/h) iterations on these systems (1,759 per Newton
// iteration on the 96^3-cell cube); a multigrid V-cycle bounds them
// independently of the mesh size.
//
// Hierarchy (built once per plan pattern and pinned set, on the host):
//   * aggregates: greedy aggregation of the free vertices over the Hessian's
//     block graph in index order (pass 1: a node whose neighbourhood is still
//     free roots an aggregate of that neighbourhood; pass 2: the rest join the
//     lowest-numbered neighbouring aggregate; pass 3: leftovers group with their
//     free neighbours), the scheme of Vanek, Mandel & Brezina (1996);
//   * tentative prolongator: per aggregate, the six rigid-body modes of
//     elasticity (translations, rotations about the mesh centroid) restricted
//     to its members, orthonormalised (modified Gram-Schmidt, twice); the
//     triangular factor R carries the modes to the next level. A mode that an
//     aggregate cannot represent (collinear members) becomes an exactly-zero
//     column, i.e. a coarse DOF with a zero row and column ("dead"), which the
//     block inverses treat as absent;
//   * coarse patterns and, per coarse block, the ordered list of fine blocks
//     whose Galerkin products P_v^T A_vw P_w sum into it (deterministic sums).
// Levels are added until the coarsest has at most kDenseNodes nodes (solved
// by its dense inverse) or aggregation stops reducing (all nodes isolated,
// e.g. packed meshes: the coarsest is then block diagonal and its block-
// Jacobi solve is exact).
//
// Per Newton system (device): Galerkin products level by level, inverses of
// the 6x6 diagonal blocks, the coarsest dense inverse, and the largest
// eigenvalue of M A on every smoothed level by power iteration (M the level's
// smoother), from which the Chebyshev coefficients follow.
//
// V-cycle (the PCG preconditioner, symmetric): on level 0 one Chebyshev step
// of the smoother before and after the coarse correction; on coarse levels
// `deg` steps (1 on level 1, 5 below by default). The smoother of level 0 is
// block-Jacobi or the learned factor M = G^T G (the network's output on the
// Hessian's lower block pattern). The smoothing passes read exactly
// symmetric BF16 copies of the operators (the fine one in padded rows); the
// Galerkin products use the FP32 values. Every kernel becomes a no-op once
// the PCG's convergence flag is set, so fixed-length CUDA graphs of PCG
// iterations can contain it.
#include <algorithm>
#include <climits>
#include <type_traits>
#include <cmath>
#include <cstdlib>
#include <cstring>

#include "amg_internal.cuh"
#include "lpcg_internal.cuh"
#include "pcg_common.cuh"

namespace bartels {

int reduce_sum(bartels_ctx ctx, const double *in, int n, double *out);
int launch_minv_blk(bartels_ctx ctx, bartels_mesh_plan plan, const float *values, float *minv);
int plan_lanes_spmv(bartels_ctx ctx, bartels_mesh_plan plan);
int plan_lanes_tri(bartels_ctx ctx, bartels_mesh_plan plan);

namespace {

constexpr int kDenseNodes = 24;   // coarsest level solved densely up to 24 nodes (144 DOFs)
constexpr int kPowerIters = 10;   // power iterations for each smoother's largest eigenvalue
constexpr int kCoarsestDeg = 6;   // Chebyshev steps on a coarsest level that is neither dense nor block diagonal

int env_int(const char *name, int dflt, int lo, int hi) {
  const char *s = std::getenv(name);
  if (!s || !*s) return dflt;
  const int v = std::atoi(s);
  return std::min(hi, std::max(lo, v));
}

// ------------------------------------------------------------ host set-up ---
struct HostLevel {
  int n = 0, bs = 0;
  std::vector<int> rp, ci;       // block pattern
  std::vector<char> active;      // node takes part in the system
  std::vector<double> B;         // n x bs x 6 near-null space (row-major per node)
  // transfer to the next level
  std::vector<int> agg, mptr, midx, gptr;
  std::vector<int2> gent;
  std::vector<float> Q;          // n x bs x 6
  int nc = 0;
};

// Greedy aggregation over the active nodes of a level, in index order.
int aggregate(const HostLevel &L, std::vector<int> &agg) {
  const int n = L.n;
  agg.assign(n, -1);
  int na = 0;
  for (int v = 0; v < n; ++v) {  // pass 1: roots with an entirely free neighbourhood
    if (!L.active[v] || agg[v] >= 0) continue;
    bool free_nb = true;
    for (int k = L.rp[v]; k < L.rp[v + 1] && free_nb; ++k) {
      const int w = L.ci[k];
      if (L.active[w] && agg[w] >= 0) free_nb = false;
    }
    if (!free_nb) continue;
    for (int k = L.rp[v]; k < L.rp[v + 1]; ++k) {
      const int w = L.ci[k];
      if (L.active[w]) agg[w] = na;
    }
    agg[v] = na++;
  }
  std::vector<int> join(n, -1);
  for (int v = 0; v < n; ++v) {  // pass 2: join the lowest-numbered neighbouring aggregate of pass 1
    if (!L.active[v] || agg[v] >= 0) continue;
    int best = INT_MAX;
    for (int k = L.rp[v]; k < L.rp[v + 1]; ++k) {
      const int w = L.ci[k];
      if (L.active[w] && agg[w] >= 0) best = std::min(best, agg[w]);
    }
    if (best != INT_MAX) join[v] = best;
  }
  for (int v = 0; v < n; ++v)
    if (join[v] >= 0) agg[v] = join[v];
  for (int v = 0; v < n; ++v) {  // pass 3: leftovers group with their free neighbours
    if (!L.active[v] || agg[v] >= 0) continue;
    for (int k = L.rp[v]; k < L.rp[v + 1]; ++k) {
      const int w = L.ci[k];
      if (L.active[w] && agg[w] < 0) agg[w] = na;
    }
    agg[v] = na++;
  }
  return na;
}

// Orthonormalise the m x 6 block Bm (row-major) of one aggregate in place:
// Bm = Qm R, modified Gram-Schmidt applied twice per column. A column whose
// remainder is below 1e-9 of the block's largest column norm is dead: its Q
// column and R row are zero.
void mgs_qr(double *Bm, int m, double R[36]) {
  for (int i = 0; i < 36; ++i) R[i] = 0.0;
  double scale = 0.0;
  for (int c = 0; c < 6; ++c) {
    double s = 0.0;
    for (int i = 0; i < m; ++i) s += Bm[6 * i + c] * Bm[6 * i + c];
    scale = std::max(scale, std::sqrt(s));
  }
  bool alive[6];
  for (int c = 0; c < 6; ++c) {
    for (int pass = 0; pass < 2; ++pass)
      for (int j = 0; j < c; ++j) {
        if (!alive[j]) continue;
        double h = 0.0;
        for (int i = 0; i < m; ++i) h += Bm[6 * i + j] * Bm[6 * i + c];
        for (int i = 0; i < m; ++i) Bm[6 * i + c] -= h * Bm[6 * i + j];
        R[6 * j + c] += h;
      }
    double s = 0.0;
    for (int i = 0; i < m; ++i) s += Bm[6 * i + c] * Bm[6 * i + c];
    s = std::sqrt(s);
    alive[c] = s > 1e-9 * scale;
    if (alive[c]) {
      for (int i = 0; i < m; ++i) Bm[6 * i + c] /= s;
      R[6 * c + c] = s;
    } else {
      for (int i = 0; i < m; ++i) Bm[6 * i + c] = 0.0;
      for (int j = 0; j < 6; ++j) R[6 * c + j] = 0.0;
    }
  }
}

// Transfer operators from level L to a new level C (nodes = aggregates).
void build_transfer(HostLevel &L, HostLevel &C) {
  const int n = L.n, bs = L.bs;
  const int na = L.nc;
  // members of each aggregate, ascending
  L.mptr.assign(na + 1, 0);
  for (int v = 0; v < n; ++v)
    if (L.agg[v] >= 0) L.mptr[L.agg[v] + 1]++;
  for (int a = 0; a < na; ++a) L.mptr[a + 1] += L.mptr[a];
  L.midx.assign(L.mptr[na], 0);
  {
    std::vector<int> fill(L.mptr.begin(), L.mptr.end() - 1);
    for (int v = 0; v < n; ++v)
      if (L.agg[v] >= 0) L.midx[fill[L.agg[v]]++] = v;
  }
  // tentative prolongator blocks and the coarse near-null space
  L.Q.assign((size_t)n * bs * 6, 0.f);
  C.n = na;
  C.bs = 6;
  C.B.assign((size_t)na * 36, 0.0);
  C.active.assign(na, 1);
  std::vector<double> Bm;
  for (int a = 0; a < na; ++a) {
    const int m0 = L.mptr[a], m1 = L.mptr[a + 1];
    const int rows = (m1 - m0) * bs;
    Bm.assign((size_t)rows * 6, 0.0);
    for (int i = m0; i < m1; ++i) {
      const int v = L.midx[i];
      std::memcpy(&Bm[(size_t)(i - m0) * bs * 6], &L.B[(size_t)v * bs * 6], sizeof(double) * bs * 6);
    }
    double R[36];
    mgs_qr(Bm.data(), rows, R);
    for (int i = m0; i < m1; ++i) {
      const int v = L.midx[i];
      for (int e = 0; e < bs * 6; ++e) L.Q[(size_t)v * bs * 6 + e] = (float)Bm[(size_t)(i - m0) * bs * 6 + e];
    }
    std::memcpy(&C.B[(size_t)a * 36], R, sizeof(R));
  }
  // coarse pattern: aggregates connected by a fine block between active nodes
  C.rp.assign(na + 1, 0);
  C.ci.clear();
  std::vector<int> mark(na, -1), cols;
  for (int a = 0; a < na; ++a) {
    cols.clear();
    for (int i = L.mptr[a]; i < L.mptr[a + 1]; ++i) {
      const int v = L.midx[i];
      for (int k = L.rp[v]; k < L.rp[v + 1]; ++k) {
        const int w = L.ci[k];
        if (!L.active[w]) continue;
        const int b = L.agg[w];
        if (mark[b] != a) {
          mark[b] = a;
          cols.push_back(b);
        }
      }
    }
    std::sort(cols.begin(), cols.end());
    C.ci.insert(C.ci.end(), cols.begin(), cols.end());
    C.rp[a + 1] = (int)C.ci.size();
  }
  // Galerkin contributions per coarse block: members ascending, their blocks ascending
  const int64_t ncb = C.rp[na];
  L.gptr.assign(ncb + 1, 0);
  auto coarse_pos = [&](int a, int b) {
    return (int)(std::lower_bound(C.ci.begin() + C.rp[a], C.ci.begin() + C.rp[a + 1], b) - C.ci.begin());
  };
  for (int a = 0; a < na; ++a)
    for (int i = L.mptr[a]; i < L.mptr[a + 1]; ++i) {
      const int v = L.midx[i];
      for (int k = L.rp[v]; k < L.rp[v + 1]; ++k) {
        const int w = L.ci[k];
        if (L.active[w]) L.gptr[coarse_pos(a, L.agg[w]) + 1]++;
      }
    }
  for (int64_t b = 0; b < ncb; ++b) L.gptr[b + 1] += L.gptr[b];
  L.gent.assign(L.gptr[ncb], int2{0, 0});
  std::vector<int> fill(L.gptr.begin(), L.gptr.end() - 1);
  for (int a = 0; a < na; ++a)
    for (int i = L.mptr[a]; i < L.mptr[a + 1]; ++i) {
      const int v = L.midx[i];
      for (int k = L.rp[v]; k < L.rp[v + 1]; ++k) {
        const int w = L.ci[k];
        if (L.active[w]) L.gent[fill[coarse_pos(a, L.agg[w])]++] = int2{v, k};
      }
    }
}

template <class T>
int upload(MgHierarchy *mg, T **dst, const std::vector<T> &src) {
  *dst = nullptr;
  if (src.empty()) return BARTELS_OK;
  void *p = nullptr;
  BT_CUDA(cudaMalloc(&p, sizeof(T) * src.size()));
  mg->allocs.push_back(p);
  BT_CUDA(cudaMemcpy(p, src.data(), sizeof(T) * src.size(), cudaMemcpyHostToDevice));
  *dst = static_cast<T *>(p);
  return BARTELS_OK;
}

int dalloc(MgHierarchy *mg, void **dst, size_t bytes) {
  *dst = nullptr;
  if (bytes == 0) return BARTELS_OK;
  BT_CUDA(cudaMalloc(dst, (bytes + 255) & ~size_t(255)));
  mg->allocs.push_back(*dst);
  return BARTELS_OK;
}

template <class T>
int dalloc_n(MgHierarchy *mg, T **dst, size_t count) {
  void *p = nullptr;
  BT_CHECK(dalloc(mg, &p, sizeof(T) * count));
  *dst = static_cast<T *>(p);
  return BARTELS_OK;
}

}  // namespace

MgHierarchy::~MgHierarchy() {
  for (void *p : allocs) cudaFree(p);
}

// Build the hierarchy of the plan's pattern for its current pinned set (kept
// while the pinned set is unchanged).
int mg_prepare(bartels_ctx ctx, bartels_mesh_plan plan) {
  if (plan->mg && plan->mg->pinned_gen == plan->pinned_gen) return BARTELS_OK;
  delete plan->mg;
  plan->mg = nullptr;
  BT_CUDA(cudaStreamSynchronize(ctx->stream));
  const int nV = plan->nV;
  std::vector<unsigned char> pinned(nV, 0);
  if (plan->pinned) BT_CUDA(cudaMemcpy(pinned.data(), plan->pinned, nV, cudaMemcpyDeviceToHost));
  std::vector<double> X(3 * (size_t)nV);
  BT_CUDA(cudaMemcpy(X.data(), plan->X, sizeof(double) * X.size(), cudaMemcpyDeviceToHost));

  std::vector<HostLevel> H(1);
  HostLevel &L0 = H[0];
  L0.n = nV;
  L0.bs = 3;
  L0.rp = plan->h_brp;
  L0.ci = plan->h_bcol;
  L0.active.assign(nV, 1);
  int nfree = 0;
  double cx = 0, cy = 0, cz = 0;
  for (int v = 0; v < nV; ++v) {
    L0.active[v] = pinned[v] ? 0 : 1;
    if (L0.active[v]) {
      nfree++;
      cx += X[3 * v];
      cy += X[3 * v + 1];
      cz += X[3 * v + 2];
    }
  }
  if (nfree == 0) return fail(BARTELS_E_UNSUPPORTED, "multigrid: every vertex is pinned");
  cx /= nfree;
  cy /= nfree;
  cz /= nfree;
  // rigid-body modes of level 0: translations and rotations about the centroid
  // (theta x (x - c) = -[x - c]_x theta)
  L0.B.assign((size_t)nV * 18, 0.0);
  for (int v = 0; v < nV; ++v) {
    const double dx = X[3 * v] - cx, dy = X[3 * v + 1] - cy, dz = X[3 * v + 2] - cz;
    double *b = &L0.B[(size_t)v * 18];
    b[0] = 1; b[7] = 1; b[14] = 1;                 // translations
    b[3] = 0;   b[4] = dz;  b[5] = -dy;            // row x: (theta x d)_x = ty dz - tz dy
    b[9] = -dz; b[10] = 0;  b[11] = dx;            // row y
    b[15] = dy; b[16] = -dx; b[17] = 0;            // row z
  }
  int coarse_blockdiag = 0, dense = 0;
  for (int l = 0; l + 1 < kMgMaxLevels; ++l) {
    HostLevel &L = H[l];
    int nact = 0;
    for (int v = 0; v < L.n; ++v) nact += L.active[v];
    if (l > 0 && nact <= kDenseNodes) {
      dense = 1;
      break;
    }
    std::vector<int> agg;
    const int na = aggregate(L, agg);
    if (na >= nact) {  // no reduction: every node is isolated (block-diagonal level)
      coarse_blockdiag = 1;
      for (int v = 0; v < L.n && coarse_blockdiag; ++v)
        for (int k = L.rp[v]; k < L.rp[v + 1]; ++k)
          if (L.ci[k] != v && L.active[L.ci[k]]) {
            coarse_blockdiag = 0;
            break;
          }
      break;
    }
    L.agg = std::move(agg);
    L.nc = na;
    H.emplace_back();
    build_transfer(H[l], H[l + 1]);
  }
  if (H.size() < 2) return fail(BARTELS_E_UNSUPPORTED, "multigrid: the system is too small for a coarse level");

  auto *mg = new MgHierarchy();
  plan->mg = mg;
  mg->pinned_gen = plan->pinned_gen;
  mg->dense = dense;
  mg->coarse_blockdiag = dense ? 0 : coarse_blockdiag;
  const int deg0 = env_int("BARTELS_MG_DEG0", 1, 1, 1);
  // Chebyshev degrees: level 1 (the largest coarse level; its one step is
  // fused into the restriction) and the levels below it, whose steps are
  // cheap and cut the PCG iterations. n = 96, one multigrid solve: level 1 at
  // 3 with 3 / 4 / 5 / 6 below gives 70 / 66 / 63 / 62 iterations and 50.4 /
  // 49.5 / 49.1 / 50.1 ms; with 5 below, level 1 at 1 / 2 / 3 / 4 gives
  // 47.1 / 48.2 / 48.8 / 50.2 ms.
  const int degc = env_int("BARTELS_MG_DEGC", 1, 1, (kMgCoef - 1) / 2 + 1);
  const int degc2 = env_int("BARTELS_MG_DEGC2", 5, 1, (kMgCoef - 1) / 2 + 1);
  mg->lv.resize(H.size());
  for (size_t l = 0; l < H.size(); ++l) {
    HostLevel &h = H[l];
    MgLevel &d = mg->lv[l];
    d.n = h.n;
    d.bs = h.bs;
    d.deg = l == 0 ? deg0 : (l + 1 == H.size() ? kCoarsestDeg : (l == 1 ? degc : degc2));
    d.nc = h.nc;
    if (l > 0) {
      d.nnzb = h.rp[h.n];
      mg->coarse_nnz += 36 * d.nnzb;
      std::vector<int> dpos(h.n, -1);
      for (int v = 0; v < h.n; ++v)
        for (int k = h.rp[v]; k < h.rp[v + 1]; ++k)
          if (h.ci[k] == v) dpos[v] = k;
      for (int v = 0; v < h.n; ++v)
        if (dpos[v] < 0) return fail(BARTELS_E_DEVICE, "multigrid: coarse level without a diagonal block");
      BT_CHECK(upload(mg, &d.rp, h.rp));
      BT_CHECK(upload(mg, &d.ci, h.ci));
      BT_CHECK(upload(mg, &d.dpos, dpos));
      BT_CHECK(dalloc_n(mg, &d.val, 36 * (size_t)d.nnzb));
      BT_CHECK(dalloc_n(mg, &d.val16, 36 * (size_t)d.nnzb));
      BT_CHECK(dalloc_n(mg, &d.dinv, 36 * (size_t)d.n));
      // position of block (J, I) for each block (I, J) (Galerkin patterns are symmetric)
      std::vector<int> rev(d.nnzb, -1);
      for (int v = 0; v < h.n; ++v)
        for (int k = h.rp[v]; k < h.rp[v + 1]; ++k) {
          const int w = h.ci[k];
          const int *b = h.ci.data() + h.rp[w], *e = h.ci.data() + h.rp[w + 1];
          const int *f = std::lower_bound(b, e, v);
          if (f == e || *f != v) return fail(BARTELS_E_DEVICE, "multigrid: coarse pattern is not symmetric");
          rev[k] = (int)(f - h.ci.data());
        }
      BT_CHECK(upload(mg, &d.rev, rev));
    } else {
      d.nnzb = plan->nnzb;
    }
    if (l + 1 < H.size()) {
      BT_CHECK(upload(mg, &d.agg, h.agg));
      BT_CHECK(upload(mg, &d.mptr, h.mptr));
      BT_CHECK(upload(mg, &d.midx, h.midx));
      BT_CHECK(upload(mg, &d.Q, h.Q));
      BT_CHECK(upload(mg, &d.gptr, h.gptr));
      BT_CHECK(upload(mg, &d.gent, h.gent));
    }
    const size_t nv = (size_t)d.bs * d.n;
    if (l > 0) BT_CHECK(dalloc_n(mg, &d.b, nv));
    BT_CHECK(dalloc_n(mg, &d.x, nv));
    BT_CHECK(dalloc_n(mg, &d.x2, nv));
    BT_CHECK(dalloc_n(mg, &d.r, nv));
    BT_CHECK(dalloc_n(mg, &d.d, nv));
    if (l > 0) BT_CHECK(dalloc_n(mg, &d.d2, nv));
  }
  if (env_int("BARTELS_MG_FINE_BF16", 1, 0, 1)) {
    std::vector<int> off(plan->nV + 1, 0);
    for (int v = 0; v < plan->nV; ++v) {
      const int64_t next = off[v] + 3ll * padded_row(plan->h_brp[v + 1] - plan->h_brp[v]);
      if (next > INT_MAX) return fail(BARTELS_E_UNSUPPORTED, "multigrid: BF16 copy larger than 2^31 entries");
      off[v + 1] = (int)next;
    }
    BT_CHECK(upload(mg, &mg->a16_off, off));
    BT_CHECK(dalloc_n(mg, &mg->a16, (size_t)off[plan->nV] + 4));
    // the pads stay zero (the conversion writes only the entries)
    BT_CUDA(cudaMemset(mg->a16, 0, sizeof(__nv_bfloat16) * ((size_t)off[plan->nV] + 4)));
  }
  if (mg->dense) {
    mg->nd = 6 * mg->lv.back().n;
    BT_CHECK(dalloc_n(mg, &mg->ainv, (size_t)mg->nd * mg->nd));
  }
  BT_CHECK(dalloc_n(mg, &mg->coef, (size_t)kMgMaxLevels * kMgCoef));
  BT_CHECK(dalloc_n(mg, &mg->norms, 2 * (size_t)kMgMaxLevels));
  mg->nparts = 4096;
  BT_CHECK(dalloc_n(mg, &mg->part, (size_t)mg->nparts));
  BT_CUDA(cudaMemset(mg->coef, 0, sizeof(float) * kMgMaxLevels * kMgCoef));
  return BARTELS_OK;
}

// ===================================================== numeric set-up ======
// Galerkin kernels: a group of kGalLanes consecutive lanes per coarse block;
// lane l of the group takes the block's contributions l, l + kGalLanes, ...
// in list order, and the group's partial sums are combined by a fixed
// butterfly, so each coarse entry is summed in the same order on every run.
// The heavy blocks (a diagonal block sums every pair of its aggregate's
// members, ~400 contributions at n = 96) no longer hold up a whole warp.
constexpr int kGalLanes = 8;
#define GAL_GROUP_LOOP_BEGIN                                                                       \
  const int gl = threadIdx.x % kGalLanes;                                                          \
  const int64_t gid = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / kGalLanes;                \
  const int64_t ngroups = ((int64_t)gridDim.x * blockDim.x) / kGalLanes;                           \
  for (int64_t b0 = gid - gid % (32 / kGalLanes); b0 < ncb; b0 += ngroups) {                        \
    const int64_t b = b0 + gid % (32 / kGalLanes);                                                 \
    const bool active = b < ncb;
#define GAL_GROUP_LOOP_END }

// butterfly sum over the group (every lane of the warp takes part), then the
// group's lanes store the block's 9 float4s round-robin
__device__ __forceinline__ void gal_group_store(float C[36], bool active, int gl, float *__restrict__ out) {
#pragma unroll
  for (int o = kGalLanes / 2; o > 0; o >>= 1)
#pragma unroll
    for (int i = 0; i < 36; ++i) C[i] += __shfl_xor_sync(0xffffffffu, C[i], o);
  if (active) {
    float4 *o4 = reinterpret_cast<float4 *>(out);
#pragma unroll
    for (int i = 0; i < 9; ++i)
      if (i % kGalLanes == gl) o4[i] = make_float4(C[4 * i], C[4 * i + 1], C[4 * i + 2], C[4 * i + 3]);
  }
}

// Galerkin product level 0 -> 1: C_IJ = sum over the block's contributions
// (v, k) of Q_v^T A_vw Q_w, A_vw read from the plan's value layout (row 3v+a
// of block row v holds its blocks' columns contiguously). One thread per
// coarse block, contributions summed in list order.
__global__ void __launch_bounds__(128)
k_mg_gal0(int64_t ncb, const int *__restrict__ gptr, const int2 *__restrict__ gent, const int *__restrict__ brp,
          const int *__restrict__ bcol, const float *__restrict__ val, const float *__restrict__ Q,
          float *__restrict__ cval) {
  GAL_GROUP_LOOP_BEGIN
    float C[36];
#pragma unroll
    for (int i = 0; i < 36; ++i) C[i] = 0.f;
    const int e1 = active ? gptr[b + 1] : 0;
    for (int e = (active ? gptr[b] : 0) + gl; e < e1; e += kGalLanes) {
      const int2 g = __ldg(gent + e);
      const int v = g.x, k = g.y;
      const int rb = __ldg(brp + v), rs = 3 * (__ldg(brp + v + 1) - rb);
      const int w = __ldg(bcol + k);
      const float *a0 = val + 9ll * rb + 3 * (k - rb);
      float A[9];
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int c = 0; c < 3; ++c) A[3 * a + c] = __ldg(a0 + a * rs + c);
      const float *qw = Q + 18ll * w;
      float T[18];  // A Q_w (3 x 6)
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int c = 0; c < 6; ++c)
          T[6 * a + c] = A[3 * a] * __ldg(qw + c) + A[3 * a + 1] * __ldg(qw + 6 + c) + A[3 * a + 2] * __ldg(qw + 12 + c);
      const float *qv = Q + 18ll * v;
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        float q[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) q[c] = __ldg(qv + 6 * a + c);
#pragma unroll
        for (int c = 0; c < 6; ++c)
#pragma unroll
          for (int d = 0; d < 6; ++d) C[6 * c + d] += q[c] * T[6 * a + d];
      }
    }
    gal_group_store(C, active, gl, cval + 36 * b);
  GAL_GROUP_LOOP_END
}

// Galerkin product between coarse levels (6x6 blocks, 6x6 prolongator blocks).
__global__ void __launch_bounds__(128)
k_mg_galc(int64_t ncb, const int *__restrict__ gptr, const int2 *__restrict__ gent, const int *__restrict__ ci,
          const float *__restrict__ val, const float *__restrict__ Q, float *__restrict__ cval) {
  GAL_GROUP_LOOP_BEGIN
    float C[36];
#pragma unroll
    for (int i = 0; i < 36; ++i) C[i] = 0.f;
    const int e1 = active ? gptr[b + 1] : 0;
    for (int e = (active ? gptr[b] : 0) + gl; e < e1; e += kGalLanes) {
      const int2 g = __ldg(gent + e);
      const int v = g.x, k = g.y;
      const int w = __ldg(ci + k);
      const float *A = val + 36ll * k;
      const float *qw = Q + 36ll * w;
      float T[36];  // A Q_w
#pragma unroll
      for (int a = 0; a < 6; ++a) {
        float ar[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) ar[c] = __ldg(A + 6 * a + c);
#pragma unroll
        for (int d = 0; d < 6; ++d) {
          float s = 0.f;
#pragma unroll
          for (int c = 0; c < 6; ++c) s += ar[c] * __ldg(qw + 6 * c + d);
          T[6 * a + d] = s;
        }
      }
      const float *qv = Q + 36ll * v;
#pragma unroll
      for (int a = 0; a < 6; ++a) {
        float q[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) q[c] = __ldg(qv + 6 * a + c);
#pragma unroll
        for (int c = 0; c < 6; ++c)
#pragma unroll
          for (int d = 0; d < 6; ++d) C[6 * c + d] += q[c] * T[6 * a + d];
      }
    }
    gal_group_store(C, active, gl, cval + 36 * b);
  GAL_GROUP_LOOP_END
}

// Inverse of each node's 6x6 diagonal block (symmetrised, FP64 Gauss-Jordan,
// FP32 storage). Dead DOFs (a zero diagonal entry: a mode the aggregate cannot
// represent) get zero rows and columns in the inverse. A block that is not
// positive definite falls back to the inverse of its diagonal.
__global__ void k_mg_inv6(int n, const int *__restrict__ dpos, const float *__restrict__ val, float *__restrict__ dinv) {
  for (int I = blockIdx.x * blockDim.x + threadIdx.x; I < n; I += gridDim.x * blockDim.x) {
    const float *a = val + 36ll * dpos[I];
    double A[36];
    bool dead[6];
    for (int i = 0; i < 6; ++i)
      for (int j = 0; j < 6; ++j) A[6 * i + j] = 0.5 * ((double)a[6 * i + j] + (double)a[6 * j + i]);
    for (int i = 0; i < 6; ++i) {
      dead[i] = !(A[7 * i] != 0.0);
      if (dead[i]) {
        for (int j = 0; j < 6; ++j) A[6 * i + j] = A[6 * j + i] = 0.0;
        A[7 * i] = 1.0;
      }
    }
    double D[36];
    for (int i = 0; i < 36; ++i) D[i] = A[i];
    bool ok = true;
    for (int k = 0; k < 6 && ok; ++k) {
      const double piv = A[7 * k];
      if (!(piv > 0.0) || !isfinite(piv)) {
        ok = false;
        break;
      }
      const double p = 1.0 / piv;
      for (int j = 0; j < 6; ++j)
        if (j != k) A[6 * k + j] *= p;
      for (int i = 0; i < 6; ++i) {
        if (i == k) continue;
        const double f = A[6 * i + k];
        for (int j = 0; j < 6; ++j)
          if (j != k) A[6 * i + j] -= f * A[6 * k + j];
      }
      for (int i = 0; i < 6; ++i)
        if (i != k) A[6 * i + k] *= -p;
      A[7 * k] = p;
    }
    float *o = dinv + 36ll * I;
    for (int i = 0; i < 6; ++i)
      for (int j = 0; j < 6; ++j) {
        double vv;
        if (ok) vv = A[6 * i + j];
        else vv = (i == j && D[7 * i] > 0.0) ? 1.0 / D[7 * i] : 0.0;
        if (dead[i] || dead[j]) vv = 0.0;
        o[6 * i + j] = (float)vv;
      }
  }
}

// Dense inverse of the coarsest level (nd = 6 x nodes <= 144): the level's
// blocks scattered into shared memory, in-place Gauss-Jordan (no pivoting, the
// matrix is SPD), dead DOFs as in k_mg_inv6. One CTA.
__global__ void __launch_bounds__(1024)
k_mg_dense_inv(int nodes, const int *__restrict__ rp, const int *__restrict__ ci, const float *__restrict__ val,
               float *__restrict__ ainv) {
  extern __shared__ float sA[];
  __shared__ float s_p;
  __shared__ unsigned char dead[6 * kDenseNodes];
  const int nd = 6 * nodes;
  for (int i = threadIdx.x; i < nd * nd; i += blockDim.x) sA[i] = 0.f;
  __syncthreads();
  for (int I = 0; I < nodes; ++I)
    for (int k = rp[I]; k < rp[I + 1]; ++k) {
      const int J = ci[k];
      for (int e = threadIdx.x; e < 36; e += blockDim.x) {
        const int a = e / 6, b = e - 6 * (e / 6);
        sA[(6 * I + a) * nd + 6 * J + b] = val[36ll * k + e];
      }
    }
  __syncthreads();
  for (int i = threadIdx.x; i < nd; i += blockDim.x) dead[i] = !(sA[i * nd + i] != 0.f);
  __syncthreads();
  for (int e = threadIdx.x; e < nd * nd; e += blockDim.x) {
    const int i = e / nd, j = e - nd * (e / nd);
    if (dead[i] || dead[j]) sA[e] = (i == j) ? 1.f : 0.f;
    else if (i > j) sA[e] = 0.5f * (sA[e] + sA[j * nd + i]);
  }
  __syncthreads();
  for (int e = threadIdx.x; e < nd * nd; e += blockDim.x) {
    const int i = e / nd, j = e - nd * (e / nd);
    if (i < j) sA[e] = sA[j * nd + i];
  }
  __syncthreads();
  for (int k = 0; k < nd; ++k) {
    if (threadIdx.x == 0) {
      const float piv = sA[k * nd + k];
      s_p = (piv > 0.f) ? 1.f / piv : 0.f;
    }
    __syncthreads();
    const float p = s_p;
    for (int j = threadIdx.x; j < nd; j += blockDim.x)
      if (j != k) sA[k * nd + j] *= p;
    __syncthreads();
    for (int e = threadIdx.x; e < nd * nd; e += blockDim.x) {
      const int i = e / nd, j = e - nd * (e / nd);
      if (i != k && j != k) sA[e] -= sA[i * nd + k] * sA[k * nd + j];
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nd; i += blockDim.x) {
      if (i != k) sA[i * nd + k] *= -p;
      else sA[k * nd + k] = p;
    }
    __syncthreads();
  }
  for (int e = threadIdx.x; e < nd * nd; e += blockDim.x) {
    const int i = e / nd, j = e - nd * (e / nd);
    ainv[e] = (dead[i] || dead[j]) ? 0.f : sA[e];
  }
}

__device__ __forceinline__ void apply_dinv6(const float *__restrict__ dinv, int I, const float r[6], float z[6]) {
  const float4 *m4 = reinterpret_cast<const float4 *>(dinv + 36ll * I);
  float m[36];
#pragma unroll
  for (int q = 0; q < 9; ++q) {
    const float4 t = __ldg(m4 + q);
    m[4 * q] = t.x; m[4 * q + 1] = t.y; m[4 * q + 2] = t.z; m[4 * q + 3] = t.w;
  }
#pragma unroll
  for (int a = 0; a < 6; ++a) {
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < 6; ++c) s += m[6 * a + c] * r[c];
    z[a] = s;
  }
}

// ============================================================= transfers ===
// b_c[I] = sum over members v of Q_v^T r_v: 8 lanes per aggregate (members
// strided over the lanes, fixed shuffle tree).
// With cdinv set it also takes the coarse level's first smoothing step from
// x = 0 (x = c Dinv b, r = b, d = x; c = ccoef[0], or 1 without ccoef).
template <int BSF>
__global__ void __launch_bounds__(256)
k_mg_restrict(int nc, const int *__restrict__ mptr, const int *__restrict__ midx, const float *__restrict__ Q,
              const float *__restrict__ r, float *__restrict__ bc, const float *__restrict__ cdinv,
              float *__restrict__ cx, float *__restrict__ cr, float *__restrict__ cd, const float *__restrict__ ccoef,
              const PcgState *__restrict__ st) {
  pdl_wait();
  pdl_trigger();
  if (st && st->done) return;
  const int lane = threadIdx.x & 31, sl = lane & 7, g = lane >> 3;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int I0 = warp * 4; I0 < nc; I0 += nwarps * 4) {
    const int I = I0 + g;
    float acc[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (I < nc) {
      const int m1 = __ldg(mptr + I + 1);
      for (int m = __ldg(mptr + I) + sl; m < m1; m += 8) {
        const int v = __ldg(midx + m);
        const float *q = Q + (int64_t)BSF * 6 * v;
#pragma unroll
        for (int a = 0; a < BSF; ++a) {
          const float rv = __ldcg(r + (int64_t)BSF * v + a);
#pragma unroll
          for (int c = 0; c < 6; ++c) acc[c] += __ldg(q + 6 * a + c) * rv;
        }
      }
    }
#pragma unroll
    for (int o = 4; o > 0; o >>= 1)
#pragma unroll
      for (int c = 0; c < 6; ++c) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], o);
    if (I < nc && sl == 0) {
#pragma unroll
      for (int c = 0; c < 6; ++c) bc[6 * I + c] = acc[c];
      if (cdinv) {
        const float cf = ccoef ? ccoef[0] : 1.f;
        float z[6];
        apply_dinv6(cdinv, I, acc, z);
#pragma unroll
        for (int c = 0; c < 6; ++c) {
          const float xv = cf * z[c];
          cx[6 * I + c] = xv;
          if (cr) cr[6 * I + c] = acc[c];
          if (cd) cd[6 * I + c] = xv;
        }
      }
    }
  }
}

// x_v += Q_v x_c[agg v] (nodes outside the system keep their value)
template <int BSF>
__global__ void __launch_bounds__(256)
k_mg_prolong(int n, const int *__restrict__ agg, const float *__restrict__ Q, const float *__restrict__ xc,
             float *__restrict__ x, const PcgState *__restrict__ st) {
  pdl_wait();
  pdl_trigger();
  if (st && st->done) return;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    const int I = __ldg(agg + v);
    if (I < 0) continue;
    float c[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) c[k] = __ldcg(xc + 6 * I + k);
    const float *q = Q + (int64_t)BSF * 6 * v;
#pragma unroll
    for (int a = 0; a < BSF; ++a) {
      float s = 0.f;
#pragma unroll
      for (int k = 0; k < 6; ++k) s += __ldg(q + 6 * a + k) * c[k];
      x[(int64_t)BSF * v + a] += s;
    }
  }
}

// ================================================= level-0 (plan layout) ===
// x = c Dinv r with the 3x3 block-Jacobi inverse (c = coef[0], or 1 without coef)
__global__ void __launch_bounds__(256)
k_mg0_bj(int nV, const float *__restrict__ minv, const float *__restrict__ r, float *__restrict__ x,
         const float *__restrict__ coef, const PcgState *__restrict__ st) {
  pdl_wait();
  pdl_trigger();
  if (st && st->done) return;
  const float c = coef ? coef[0] : 1.f;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nV; v += gridDim.x * blockDim.x) {
    float rv[3], zv[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) rv[k] = __ldcg(r + 3 * v + k);
    apply_minv(minv, v, rv, zv);
#pragma unroll
    for (int k = 0; k < 3; ++k) x[3 * v + k] = c * zv[k];
  }
}

// The PCG update fused with the level-0 pre-smoothing of the block-Jacobi
// V-cycle: x += alpha p; r -= alpha Ap; x0 = c Dinv r (c = coef[0]); partial
// sums of r.r. The last block stores r.r, advances the iteration count and
// applies the convergence test, as k_pcg_update_f does.
__global__ void __launch_bounds__(256)
k_mg0_update(int nV, const float *__restrict__ pa, const float *__restrict__ pb, const float *__restrict__ ap,
             float *__restrict__ x, float *__restrict__ r, const float *__restrict__ minv, float *__restrict__ x0,
             const float *__restrict__ coef, double *__restrict__ part, PcgState *__restrict__ st) {
  pdl_wait();
  pdl_trigger();
  if (st->done) return;
  const int it = st->it;
  const float *p = (it & 1) ? pb : pa;
  const float alpha = st->alpha, c = coef[0];
  float arr = 0.f;
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nV; v += gridDim.x * blockDim.x) {
    float rv[3], zv[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const int i = 3 * v + k;
      x[i] += alpha * __ldcg(p + i);
      rv[k] = r[i] - alpha * __ldcg(ap + i);
      r[i] = rv[k];
      arr += rv[k] * rv[k];
    }
    apply_minv(minv, v, rv, zv);
#pragma unroll
    for (int k = 0; k < 3; ++k) x0[3 * v + k] = c * zv[k];
  }
  double s = cta_sum_f(arr);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
  if (last_block(&st->count)) {
    const double rr = sum_partials(part, gridDim.x);
    if (threadIdx.x == 0) {
      st->rr = rr;
      st->it = it + 1;
      if (rr <= st->tol2 || it + 1 >= st->max_it || !(rr == rr)) st->done = 1;
      st->count = 0;
    }
  }
}

// BF16 copy of the finest level's values for the V-cycle's SpMVs, exactly
// symmetric: entry (3v+k, 3w+l) of block p = (v, w) and entry (3w+l, 3v+k) of
// its transpose q = rev[p] both take bf16((A_p(k,l) + A_q(l,k)) / 2). One warp
// per vertex row, one lane per block.
__global__ void __launch_bounds__(256)
k_mg0_to_bf16(int nV, const int *__restrict__ brp, const int *__restrict__ bcol, const int *__restrict__ rev,
              const float *__restrict__ val, const int *__restrict__ a16_off, __nv_bfloat16 *__restrict__ a16) {
  const int lane = threadIdx.x & 31;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int v = warp; v < nV; v += nwarps) {
    const int rb = brp[v], nb = brp[v + 1] - rb, rs = 3 * nb, rsp = padded_row(nb);
    __nv_bfloat16 *out = a16 + __ldg(a16_off + v);
    for (int j = lane; j < nb; j += 32) {
      const int w = __ldg(bcol + rb + j);
      const int q = __ldg(rev + rb + j);
      const int rbw = __ldg(brp + w), rsw = 3 * (__ldg(brp + w + 1) - rbw), jq = q - rbw;
#pragma unroll
      for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int l = 0; l < 3; ++l) {
          const float a = __ldg(val + 9ll * rb + k * rs + 3 * j + l);
          const float t = __ldg(val + 9ll * rbw + l * rsw + 3 * jq + k);
          out[k * rsp + 3 * j + l] = __float2bfloat16_rn(0.5f * (a + t));
        }
    }
  }
}

// One row of the finest level: the FP32 values in the plan's layout
// (off == nullptr), or the padded BF16 copy (4 values per 8-byte load).
template <int G, class VT, class XV>
__device__ __forceinline__ void row0_acc(int v, int sl, const int *__restrict__ brp, const int *__restrict__ bcol,
                                         const VT *__restrict__ val, const int *__restrict__ off, XV &&xval,
                                         float &s0, float &s1, float &s2) {
  if constexpr (std::is_same<VT, __nv_bfloat16>::value) {
    const int rb = __ldg(brp + v), nb = __ldg(brp + v + 1) - rb;
    tri_row_acc4<G>(sl, bcol + rb, val + __ldg(off + v), 3 * nb, padded_row(nb), xval, s0, s1, s2);
  } else {
    spmv_row_acc<G>(v, sl, brp, bcol, val, xval, s0, s1, s2);
  }
}

// out = b - A x, or A x without b (rows of pinned vertices give 0)
template <int G, class VT>
__global__ void __launch_bounds__(256)
k_mg0_resid(int nV, const int *__restrict__ brp, const int *__restrict__ bcol, const VT *__restrict__ val,
            const int *__restrict__ off, const float *__restrict__ b, const float *__restrict__ x,
            float *__restrict__ out, const unsigned char *__restrict__ pinned, const PcgState *__restrict__ st) {
  pdl_wait();
  pdl_trigger();
  if (st && st->done) return;
  BT_ROW_LOOP_BEGIN(G)
  float s0 = 0.f, s1 = 0.f, s2 = 0.f;
  if (active) row0_acc<G>(v, sl, brp, bcol, val, off, [&](int c) { return __ldcg(x + c); }, s0, s1, s2);
  group_reduce<G>(s0, s1, s2);
  if (active && sl == 0) {
    if (b) {
      s0 = __ldcg(b + 3 * v) - s0;
      s1 = __ldcg(b + 3 * v + 1) - s1;
      s2 = __ldcg(b + 3 * v + 2) - s2;
    }
    if (pinned && pinned[v]) s0 = s1 = s2 = 0.f;
    out[3 * v] = s0;
    out[3 * v + 1] = s1;
    out[3 * v + 2] = s2;
  }
  BT_ROW_LOOP_END
}

// Final step of the V-cycle with the block-Jacobi smoother:
// z = x + c Dinv (b - A x), partial sums of b.z; the last block stores r.z
// and beta = r.z / r.z_old in the PCG state.
template <int G, class VT>
__global__ void __launch_bounds__(256)
k_mg0_post_bj(int nV, const int *__restrict__ brp, const int *__restrict__ bcol, const VT *__restrict__ val,
              const int *__restrict__ off, const float *__restrict__ minv, const float *__restrict__ b,
              const float *__restrict__ x, float *__restrict__ z, const unsigned char *__restrict__ pinned,
              const float *__restrict__ coef, double *__restrict__ part, PcgState *__restrict__ st) {
  pdl_wait();
  pdl_trigger();
  if (st->done) return;
  const float c = coef[0];
  float acc = 0.f;
  BT_ROW_LOOP_BEGIN(G)
  float s0 = 0.f, s1 = 0.f, s2 = 0.f;
  if (active) row0_acc<G>(v, sl, brp, bcol, val, off, [&](int cc) { return __ldcg(x + cc); }, s0, s1, s2);
  group_reduce<G>(s0, s1, s2);
  if (active && sl == 0) {
    float bv[3], rv[3], zv[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) bv[k] = __ldcg(b + 3 * v + k);
    rv[0] = bv[0] - s0;
    rv[1] = bv[1] - s1;
    rv[2] = bv[2] - s2;
    apply_minv(minv, v, rv, zv);
    const bool pin = pinned && pinned[v];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const float zk = pin ? 0.f : __ldcg(x + 3 * v + k) + c * zv[k];
      z[3 * v + k] = zk;
      acc += bv[k] * zk;
    }
  }
  BT_ROW_LOOP_END
  double s = cta_sum_f(acc);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
  if (last_block(&st->count)) {
    const double rz = sum_partials(part, gridDim.x);
    if (threadIdx.x == 0) {
      st->beta = (float)(rz / st->rz);
      st->rz = rz;
      st->count = 0;
    }
  }
}

// y = G r (learned factor, lower rows; pinned rows give 0)
template <int G>
__global__ void __launch_bounds__(256)
k_mg0_fac_lower(int nV, const int4 *__restrict__ meta, const int *__restrict__ bcol,
                const __nv_bfloat16 *__restrict__ gl, const float *__restrict__ r, float *__restrict__ y,
                const unsigned char *__restrict__ pinned, const PcgState *__restrict__ st) {
  pdl_wait();
  pdl_trigger();
  if (st && st->done) return;
  BT_ROW_LOOP_BEGIN(G)
  float s0 = 0.f, s1 = 0.f, s2 = 0.f;
  if (active) {
    const int4 m = __ldg(meta + v);
    const int nl = (m.w & 0xFFFF) + 1;
    tri_row_acc4<G>(sl, bcol + m.x, gl + m.y, 3 * nl, padded_row(nl), [&](int c) { return __ldcg(r + c); }, s0, s1,
                    s2);
  }
  group_reduce<G>(s0, s1, s2);
  if (active && sl == 0) {
    if (pinned && pinned[v]) s0 = s1 = s2 = 0.f;
    y[3 * v] = s0;
    y[3 * v + 1] = s1;
    y[3 * v + 2] = s2;
  }
  BT_ROW_LOOP_END
}

// out = (xin, or 0) + c G^T y (upper rows), c = coef[0] (1 without coef). With
// b and part (the final V-cycle step) also r.z = b.out and beta in the state.
template <int G>
__global__ void __launch_bounds__(256)
k_mg0_fac_upper(int nV, const int4 *__restrict__ meta, const int *__restrict__ bcol,
                const __nv_bfloat16 *__restrict__ gu, const float *__restrict__ y, const float *__restrict__ xin,
                float *__restrict__ out, const unsigned char *__restrict__ pinned, const float *__restrict__ coef,
                const float *__restrict__ b, double *__restrict__ part, PcgState *__restrict__ st) {
  pdl_wait();
  pdl_trigger();
  if (st && st->done) return;
  const float c = coef ? coef[0] : 1.f;
  float acc = 0.f;
  BT_ROW_LOOP_BEGIN(G)
  float s0 = 0.f, s1 = 0.f, s2 = 0.f;
  if (active) {
    const int4 m = __ldg(meta + v);
    const int d = m.w & 0xFFFF, nu = (m.w >> 16) - d;
    tri_row_acc4<G>(sl, bcol + m.x + d, gu + m.z, 3 * nu, padded_row(nu), [&](int cc) { return __ldcg(y + cc); }, s0,
                    s1, s2);
  }
  group_reduce<G>(s0, s1, s2);
  if (active && sl == 0) {
    const bool pin = pinned && pinned[v];
    float o[3] = {c * s0, c * s1, c * s2};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      if (xin) o[k] += __ldcg(xin + 3 * v + k);
      if (pin) o[k] = 0.f;
      out[3 * v + k] = o[k];
      if (b) acc += __ldcg(b + 3 * v + k) * o[k];
    }
  }
  BT_ROW_LOOP_END
  if (!part) return;
  double s = cta_sum_f(acc);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
  if (last_block(&st->count)) {
    const double rz = sum_partials(part, gridDim.x);
    if (threadIdx.x == 0) {
      st->beta = (float)(rz / st->rz);
      st->rz = rz;
      st->count = 0;
    }
  }
}

// BF16 copy of a coarse level, exactly symmetric: block k gets
// (C_k + C_rev(k)^T) / 2, rounded once (C_k and C_rev(k) come from separate
// Galerkin sums and may differ in their last bits).
__global__ void __launch_bounds__(256)
k_mgc_to_bf16(int64_t nnzb, const int *__restrict__ rev, const float *__restrict__ val,
              __nv_bfloat16 *__restrict__ val16) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nnzb; k += (int64_t)gridDim.x * blockDim.x) {
    const float *a = val + 36 * k, *t = val + 36ll * __ldg(rev + k);
    __nv_bfloat16 *o = val16 + 36 * k;
#pragma unroll
    for (int r = 0; r < 6; ++r)
#pragma unroll
      for (int c = 0; c < 6; ++c)
        o[6 * r + c] = __float2bfloat16_rn(0.5f * (__ldg(a + 6 * r + c) + __ldg(t + 6 * c + r)));
  }
}

// ======================================================== coarse levels ===
// Row I of a 6x6-block level: G lanes stride the row's blocks; s = A_I. x
template <int G, class XV>
__device__ __forceinline__ void crow_acc(int I, int sl, const int *__restrict__ rp, const int *__restrict__ ci,
                                         const __nv_bfloat16 *__restrict__ val, XV &&xv, float s[6]) {
  const int k1 = __ldg(rp + I + 1);
  for (int k = __ldg(rp + I) + sl; k < k1; k += G) {
    const int J = __ldg(ci + k);
    float xj[6];
#pragma unroll
    for (int c = 0; c < 6; ++c) xj[c] = xv(6 * J + c);
    // 36 BF16 values = 9 x 8 bytes
    const uint2 *a2 = reinterpret_cast<const uint2 *>(val + 36ll * k);
    float a[36];
#pragma unroll
    for (int q = 0; q < 9; ++q) {
      const uint2 t = __ldg(a2 + q);
      a[4 * q] = __uint_as_float(t.x << 16);
      a[4 * q + 1] = __uint_as_float(t.x & 0xFFFF0000u);
      a[4 * q + 2] = __uint_as_float(t.y << 16);
      a[4 * q + 3] = __uint_as_float(t.y & 0xFFFF0000u);
    }
#pragma unroll
    for (int r = 0; r < 6; ++r)
#pragma unroll
      for (int c = 0; c < 6; ++c) s[r] += a[6 * r + c] * xj[c];
  }
}

template <int G>
__device__ __forceinline__ void group_reduce6(float s[6]) {
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1)
#pragma unroll
    for (int r = 0; r < 6; ++r) s[r] += __shfl_xor_sync(0xffffffffu, s[r], o);
}


#define BT_CROW_LOOP_BEGIN(G)                                                   \
  const int lane_ = threadIdx.x & 31, sl = lane_ % (G), gw_ = lane_ / (G);     \
  const int warp_ = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;              \
  const int nwarps_ = (gridDim.x * blockDim.x) >> 5;                           \
  for (int ib_ = warp_ * (32 / (G)); ib_ < n; ib_ += nwarps_ * (32 / (G))) {   \
    const int I = ib_ + gw_;                                                    \
    const bool active = I < n;
#define BT_CROW_LOOP_END }

// first smoothing step from x = 0: x = d = c0 Dinv b, r = b (x = Dinv b when exact)
__global__ void __launch_bounds__(256)
k_mgc_first(int n, const float *__restrict__ dinv, const float *__restrict__ b, float *__restrict__ x,
            float *__restrict__ r, float *__restrict__ d, const float *__restrict__ coef,
            const PcgState *__restrict__ st) {
  pdl_wait();
  pdl_trigger();
  if (st && st->done) return;
  const float c = coef ? coef[0] : 1.f;
  for (int I = blockIdx.x * blockDim.x + threadIdx.x; I < n; I += gridDim.x * blockDim.x) {
    float bv[6], z[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) bv[k] = __ldcg(b + 6 * I + k);
    apply_dinv6(dinv, I, bv, z);
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      const float xv = c * z[k];
      x[6 * I + k] = xv;
      if (r) r[6 * I + k] = bv[k];
      if (d) d[6 * I + k] = xv;
    }
  }
}

// Chebyshev step j >= 1: r -= A d_in; d_out = c1 d_in + c2 Dinv r; x += d_out
template <int G>
__global__ void __launch_bounds__(256)
k_mgc_cheb(int n, const int *__restrict__ rp, const int *__restrict__ ci, const __nv_bfloat16 *__restrict__ val,
           const float *__restrict__ dinv, const float *__restrict__ d_in, float *__restrict__ d_out,
           float *__restrict__ r, float *__restrict__ x, const float *__restrict__ coef, int j,
           const PcgState *__restrict__ st) {
  pdl_wait();
  pdl_trigger();
  if (st && st->done) return;
  const float c1 = coef[2 * j - 1], c2 = coef[2 * j];
  BT_CROW_LOOP_BEGIN(G)
  float s[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  if (active) crow_acc<G>(I, sl, rp, ci, val, [&](int c) { return __ldcg(d_in + c); }, s);
  group_reduce6<G>(s);
  if (active && sl == 0) {
    float rv[6], z[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      rv[k] = r[6 * I + k] - s[k];
      r[6 * I + k] = rv[k];
    }
    apply_dinv6(dinv, I, rv, z);
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      const float dk = c1 * __ldcg(d_in + 6 * I + k) + c2 * z[k];
      d_out[6 * I + k] = dk;
      x[6 * I + k] += dk;
    }
  }
  BT_CROW_LOOP_END
}

// r = b - A x
template <int G>
__global__ void __launch_bounds__(256)
k_mgc_resid(int n, const int *__restrict__ rp, const int *__restrict__ ci, const __nv_bfloat16 *__restrict__ val,
            const float *__restrict__ b, const float *__restrict__ x, float *__restrict__ r,
            const PcgState *__restrict__ st) {
  pdl_wait();
  pdl_trigger();
  if (st && st->done) return;
  BT_CROW_LOOP_BEGIN(G)
  float s[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  if (active) crow_acc<G>(I, sl, rp, ci, val, [&](int c) { return __ldcg(x + c); }, s);
  group_reduce6<G>(s);
  if (active && sl == 0)
#pragma unroll
    for (int k = 0; k < 6; ++k) r[6 * I + k] = __ldcg(b + 6 * I + k) - s[k];
  BT_CROW_LOOP_END
}

// first post-smoothing step: r = b - A x; d = c0 Dinv r; x_out = x + d
template <int G>
__global__ void __launch_bounds__(256)
k_mgc_post_first(int n, const int *__restrict__ rp, const int *__restrict__ ci, const __nv_bfloat16 *__restrict__ val,
                 const float *__restrict__ dinv, const float *__restrict__ b, const float *__restrict__ x,
                 float *__restrict__ x_out, float *__restrict__ r, float *__restrict__ d,
                 const float *__restrict__ coef, const PcgState *__restrict__ st) {
  pdl_wait();
  pdl_trigger();
  if (st && st->done) return;
  const float c0 = coef[0];
  BT_CROW_LOOP_BEGIN(G)
  float s[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  if (active) crow_acc<G>(I, sl, rp, ci, val, [&](int c) { return __ldcg(x + c); }, s);
  group_reduce6<G>(s);
  if (active && sl == 0) {
    float rv[6], z[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      rv[k] = __ldcg(b + 6 * I + k) - s[k];
      r[6 * I + k] = rv[k];
    }
    apply_dinv6(dinv, I, rv, z);
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      const float dk = c0 * z[k];
      d[6 * I + k] = dk;
      x_out[6 * I + k] = __ldcg(x + 6 * I + k) + dk;
    }
  }
  BT_CROW_LOOP_END
}

// y = Dinv (A x) (power iteration on a coarse level)
template <int G>
__global__ void __launch_bounds__(256)
k_mgc_MA(int n, const int *__restrict__ rp, const int *__restrict__ ci, const __nv_bfloat16 *__restrict__ val,
         const float *__restrict__ dinv, const float *__restrict__ x, float *__restrict__ y) {
  BT_CROW_LOOP_BEGIN(G)
  float s[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  if (active) crow_acc<G>(I, sl, rp, ci, val, [&](int c) { return __ldcg(x + c); }, s);
  group_reduce6<G>(s);
  if (active && sl == 0) {
    float z[6];
    apply_dinv6(dinv, I, s, z);
#pragma unroll
    for (int k = 0; k < 6; ++k) y[6 * I + k] = z[k];
  }
  BT_CROW_LOOP_END
}

// coarsest level, dense: x = Ainv b (one CTA)
__global__ void __launch_bounds__(256)
k_mg_dense_apply(int nd, const float *__restrict__ ainv, const float *__restrict__ b, float *__restrict__ x,
                 const PcgState *__restrict__ st) {
  pdl_wait();
  pdl_trigger();
  if (st && st->done) return;
  __shared__ float sb[6 * kDenseNodes];
  for (int i = threadIdx.x; i < nd; i += blockDim.x) sb[i] = __ldcg(b + i);
  __syncthreads();
  for (int i = threadIdx.x; i < nd; i += blockDim.x) {
    float s = 0.f;
    for (int j = 0; j < nd; ++j) s += __ldg(ainv + (int64_t)i * nd + j) * sb[j];
    x[i] = s;
  }
}

// ==================================================== eigenvalue bounds ===
// deterministic start vector in [-1, 1] (integer hash of the index)
__global__ void k_mg_hash_fill(int64_t n, float *__restrict__ v, unsigned seed) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    unsigned h = (unsigned)i * 2654435761u ^ seed;
    h ^= h >> 16;
    h *= 2246822519u;
    h ^= h >> 13;
    h *= 3266489917u;
    h ^= h >> 16;
    v[i] = (float)(h & 0xFFFFFF) * (2.f / 16777215.f) - 1.f;
  }
}

__global__ void __launch_bounds__(256) k_mg_sumsq(int64_t n, const float *__restrict__ v, double *__restrict__ part) {
  float acc = 0.f;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float t = v[i];
    acc += t * t;
  }
  double s = cta_sum_f(acc);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// Packed meshes: squared norms of v over each segment's DOFs (one CTA per
// segment, fixed order)
__global__ void __launch_bounds__(256)
k_mg_seg_sumsq(const int *__restrict__ voff, const float *__restrict__ v, double *__restrict__ out) {
  const int s = blockIdx.x;
  float acc = 0.f;
  for (int i = 3 * voff[s] + threadIdx.x; i < 3 * voff[s + 1]; i += blockDim.x) {
    const float t = v[i];
    acc += t * t;
  }
  const double r = cta_sum_f(acc);
  if (threadIdx.x == 0) out[s] = r;
}

// The power iteration of a block-diagonal operator runs independently in each
// block, so the per-segment norm ratios estimate every segment's own largest
// eigenvalue; their maximum bounds all of them (a ratio over the whole vector
// is dominated by the largest segments and can miss a small stiff one).
// Written as norms (1, max ratio) for k_mg_coef.
__global__ void k_mg_seg_lmax(int nseg, const double *__restrict__ prev, const double *__restrict__ last,
                              double *__restrict__ norms) {
  double m = 0.0;
  for (int s = threadIdx.x; s < nseg; s += blockDim.x)
    if (prev[s] > 0.0 && last[s] > 0.0 && isfinite(last[s])) m = fmax(m, last[s] / prev[s]);
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if (threadIdx.x == 0) {
    norms[0] = 1.0;
    norms[1] = m > 0.0 ? m : 1.0;
  }
}

struct MgDegrees {
  int deg[kMgMaxLevels];
  int nlev;
};

// Chebyshev coefficients of each smoothed level from its power-iteration
// norms: lambda_max = 1.1 |y_K| / |y_{K-1}|, interval [lambda_max / 10,
// lambda_max]; coef = {1/theta, (c1_j, c2_j) for j = 1 .. deg-1} with
// rho_0 = delta/theta, rho_j = 1/(2 sigma - rho_{j-1}), c1_j = rho_j rho_{j-1},
// c2_j = 2 rho_j / delta (the Chebyshev semi-iteration, Saad 2003, Alg. 12.1).
__global__ void k_mg_coef(MgDegrees dg, const double *__restrict__ norms, float *__restrict__ coef) {
  const int l = threadIdx.x;
  if (l >= dg.nlev) return;
  const double a = norms[2 * l], b = norms[2 * l + 1];
  double lmax = (a > 0.0 && b > 0.0 && isfinite(a) && isfinite(b)) ? 1.1 * sqrt(b / a) : 1.0;
  const double lmin = lmax / 10.0;
  const double theta = 0.5 * (lmax + lmin), delta = 0.5 * (lmax - lmin), sigma = theta / delta;
  float *c = coef + kMgCoef * l;
  c[0] = (float)(1.0 / theta);
  double rho = 1.0 / sigma;
  for (int j = 1; j < dg.deg[l] && 2 * j < kMgCoef; ++j) {
    const double rn = 1.0 / (2.0 * sigma - rho);
    c[2 * j - 1] = (float)(rn * rho);
    c[2 * j] = (float)(2.0 * rn / delta);
    rho = rn;
  }
}

// ================================================================= host ====
namespace {

constexpr int kGc = 8;  // lanes per row on coarse levels

int grid_n(bartels_ctx ctx, int64_t n, int per_block = 256) {
  const int64_t g = (n + per_block - 1) / per_block;
  return (int)std::max<int64_t>(1, std::min<int64_t>(g, (int64_t)ctx->num_sms * 8));
}
// rows walked by groups of G lanes, 8 warps per 256-thread block
int grid_rows(bartels_ctx ctx, int64_t rows, int G) {
  const int64_t warps = (rows * G + 31) / 32;
  const int64_t g = (warps + 7) / 8;
  return (int)std::max<int64_t>(1, std::min<int64_t>(g, (int64_t)ctx->num_sms * 8));
}

// result vector of a level after its part of the V-cycle
float *level_result(const MgHierarchy *mg, int l) {
  const bool coarsest = l + 1 == (int)mg->lv.size();
  return coarsest ? mg->lv[l].x : mg->lv[l].x2;
}

// Chebyshev smoothing of a coarse level from x = 0 (deg steps): x, r, d. The
// first step is skipped when the restriction into the level has taken it.
int cheb_from_zero(bartels_ctx ctx, const MgLevel &c, const float *coef, bool first_done, const PcgState *st) {
  const int gr = grid_rows(ctx, c.n, kGc);
  if (!first_done)
    BT_LAUNCH_PDL(ctx, k_mgc_first, grid_n(ctx, c.n), 256, 0, c.n, c.dinv, c.b, c.x, c.r, c.d, coef, st);
  float *dc = c.d, *dn = c.d2;
  for (int j = 1; j < c.deg; ++j) {
    BT_LAUNCH_PDL(ctx, k_mgc_cheb<kGc>, gr, 256, 0, c.n, c.rp, c.ci, c.val16, c.dinv, dc, dn, c.r, c.x, coef, j, st);
    std::swap(dc, dn);
  }
  return BARTELS_OK;
}

// Restriction into level l (from level l - 1's residual r with its transfer
// blocks), taking level l's first smoothing step in the same kernel where that
// step is local (every level but a dense coarsest). Returns whether it did.
template <int BSF>
int restrict_into(bartels_ctx ctx, MgHierarchy *mg, const MgLevel &f, const float *r, int l, const PcgState *st,
                  bool *first_done) {
  MgLevel &c = mg->lv[l];
  const bool last = l + 1 == (int)mg->lv.size();
  const bool fuse = !(last && mg->dense);
  const bool exact = last && mg->coarse_blockdiag;  // x = Dinv b
  const float *coef = exact ? nullptr : mg->coef + kMgCoef * l;
  const int g = grid_rows(ctx, (c.n + 3) / 4, 32);
  if (fuse)
    BT_LAUNCH_PDL(ctx, k_mg_restrict<BSF>, g, 256, 0, c.n, f.mptr, f.midx, f.Q, r, c.b, (const float *)c.dinv, c.x,
              exact ? (float *)nullptr : c.r, exact ? (float *)nullptr : c.d, coef, st);
  else
    BT_LAUNCH_PDL(ctx, k_mg_restrict<BSF>, g, 256, 0, c.n, f.mptr, f.midx, f.Q, r, c.b, (const float *)nullptr,
              (float *)nullptr, (float *)nullptr, (float *)nullptr, (const float *)nullptr, st);
  *first_done = fuse;
  return BARTELS_OK;
}

int enqueue_coarse(bartels_ctx ctx, MgHierarchy *mg, int l, bool first_done, const PcgState *st) {
  MgLevel &c = mg->lv[l];
  const float *coef = mg->coef + kMgCoef * l;
  const int last = (int)mg->lv.size() - 1;
  if (l == last) {
    if (mg->dense) {
      BT_LAUNCH_PDL(ctx, k_mg_dense_apply, 1, 256, 0, mg->nd, mg->ainv, c.b, c.x, st);
    } else if (mg->coarse_blockdiag) {
      if (!first_done)
        BT_LAUNCH_PDL(ctx, k_mgc_first, grid_n(ctx, c.n), 256, 0, c.n, c.dinv, c.b, c.x, (float *)nullptr,
                  (float *)nullptr, (const float *)nullptr, st);
    } else {
      BT_CHECK(cheb_from_zero(ctx, c, coef, first_done, st));
    }
    return BARTELS_OK;
  }
  const int gr = grid_rows(ctx, c.n, kGc);
  BT_CHECK(cheb_from_zero(ctx, c, coef, first_done, st));
  BT_LAUNCH_PDL(ctx, k_mgc_resid<kGc>, gr, 256, 0, c.n, c.rp, c.ci, c.val16, c.b, c.x, c.r, st);
  bool next_first = false;
  BT_CHECK(restrict_into<6>(ctx, mg, c, c.r, l + 1, st, &next_first));
  BT_CHECK(enqueue_coarse(ctx, mg, l + 1, next_first, st));
  BT_LAUNCH_PDL(ctx, k_mg_prolong<6>, grid_n(ctx, c.n), 256, 0, c.n, c.agg, c.Q, level_result(mg, l + 1), c.x, st);
  BT_LAUNCH_PDL(ctx, k_mgc_post_first<kGc>, gr, 256, 0, c.n, c.rp, c.ci, c.val16, c.dinv, c.b, c.x, c.x2, c.r, c.d, coef,
            st);
  float *dc = c.d, *dn = c.d2;
  for (int j = 1; j < c.deg; ++j) {
    BT_LAUNCH_PDL(ctx, k_mgc_cheb<kGc>, gr, 256, 0, c.n, c.rp, c.ci, c.val16, c.dinv, dc, dn, c.r, c.x2, coef, j, st);
    std::swap(dc, dn);
  }
  return BARTELS_OK;
}

// level-0 launches for the plan's SpMV lane count (4, 8 or 16) or factor lane count (4 or 8)
#define BT_MG_G(G_, ...)                \
  do {                                  \
    if ((G_) == 4) {                    \
      constexpr int GL = 4;             \
      __VA_ARGS__;                      \
    } else if ((G_) == 16) {            \
      constexpr int GL = 16;            \
      __VA_ARGS__;                      \
    } else {                            \
      constexpr int GL = 8;             \
      __VA_ARGS__;                      \
    }                                   \
  } while (0)

int fac_lower(bartels_ctx ctx, bartels_mesh_plan plan, const MgSmoother &sm, const float *in, float *out,
              const PcgState *st) {
  const int GT = plan_lanes_tri(ctx, plan) == 8 ? 8 : 4;
  const int g = grid_rows(ctx, plan->nV, GT);
  BT_MG_G(GT, BT_LAUNCH_PDL(ctx, k_mg0_fac_lower<GL>, g, 256, 0, plan->nV, sm.fp->meta, plan->bcol, sm.gl, in, out,
                        plan->pinned, st));
  return BARTELS_OK;
}

int fac_upper(bartels_ctx ctx, bartels_mesh_plan plan, const MgSmoother &sm, const float *y, const float *xin,
              float *out, const float *coef, const float *b, double *part, PcgState *st) {
  const int GT = plan_lanes_tri(ctx, plan) == 8 ? 8 : 4;
  const int g = grid_rows(ctx, plan->nV, GT);
  BT_MG_G(GT, BT_LAUNCH_PDL(ctx, k_mg0_fac_upper<GL>, g, 256, 0, plan->nV, sm.fp->meta, plan->bcol, sm.gu, y, xin, out,
                        plan->pinned, coef, b, part, st));
  return BARTELS_OK;
}

// out = b - A x on the finest level, with the V-cycle's BF16 copy of A when it has one
int resid0(bartels_ctx ctx, bartels_mesh_plan plan, const float *values, const float *b, const float *x, float *out,
           const PcgState *st) {
  using B16 = __nv_bfloat16;
  const B16 *a16 = plan->mg ? plan->mg->a16 : nullptr;
  if (a16) {
    // padded BF16 rows: the factor passes' lane count (4 values per lane step)
    const int G = plan_lanes_tri(ctx, plan);
    const int g = grid_rows(ctx, plan->nV, G);
    BT_MG_G(G, BT_LAUNCH_PDL(ctx, (k_mg0_resid<GL, B16>), g, 256, 0, plan->nV, plan->brp, plan->bcol, a16,
                             (const int *)plan->mg->a16_off, b, x, out, plan->pinned, st));
  } else {
    const int G = plan_lanes_spmv(ctx, plan);
    const int g = grid_rows(ctx, plan->nV, G);
    BT_MG_G(G, BT_LAUNCH_PDL(ctx, (k_mg0_resid<GL, float>), g, 256, 0, plan->nV, plan->brp, plan->bcol, values,
                             (const int *)nullptr, b, x, out, plan->pinned, st));
  }
  return BARTELS_OK;
}

int sumsq_into(bartels_ctx ctx, MgHierarchy *mg, int64_t n, const float *v, double *out) {
  const int g = std::min(grid_n(ctx, n), mg->nparts);
  BT_LAUNCH(ctx, k_mg_sumsq, g, 256, 0, n, v, mg->part);
  return reduce_sum(ctx, mg->part, g, out);
}

}  // namespace

void mg_destroy(MgHierarchy *mg) { delete mg; }

int mg_setup_numeric(bartels_ctx ctx, bartels_mesh_plan plan, const float *values, const MgSmoother &sm) {
  MgHierarchy *mg = plan->mg;
  if (!mg) return fail(BARTELS_E_INVALID_ARG, "multigrid: no hierarchy");
  const int L = (int)mg->lv.size();
  if (mg->a16) {
    FactorPattern *fp = nullptr;
    BT_CHECK(plan_factor_pattern(plan, &fp));
    BT_LAUNCH(ctx, k_mg0_to_bf16, grid_rows(ctx, plan->nV, 32), 256, 0, plan->nV, plan->brp, plan->bcol, fp->rev,
              values, (const int *)mg->a16_off, mg->a16);
  }
  for (int l = 0; l + 1 < L; ++l) {
    MgLevel &f = mg->lv[l], &c = mg->lv[l + 1];
    const int g = grid_n(ctx, c.nnzb * kGalLanes, 128);  // kGalLanes lanes per coarse block
    if (l == 0)
      BT_LAUNCH(ctx, k_mg_gal0, g, 128, 0, c.nnzb, f.gptr, f.gent, plan->brp, plan->bcol, values, f.Q, c.val);
    else
      BT_LAUNCH(ctx, k_mg_galc, g, 128, 0, c.nnzb, f.gptr, f.gent, f.ci, f.val, f.Q, c.val);
    BT_LAUNCH(ctx, k_mg_inv6, grid_n(ctx, c.n, 128), 128, 0, c.n, c.dpos, c.val, c.dinv);
    BT_LAUNCH(ctx, k_mgc_to_bf16, grid_n(ctx, c.nnzb), 256, 0, c.nnzb, (const int *)c.rev, (const float *)c.val,
              c.val16);
  }
  if (mg->dense) {
    const MgLevel &c = mg->lv[L - 1];
    const size_t smem = sizeof(float) * mg->nd * mg->nd;
    BT_CUDA(cudaFuncSetAttribute(k_mg_dense_inv, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    BT_LAUNCH(ctx, k_mg_dense_inv, 1, 1024, smem, c.n, c.rp, c.ci, c.val, mg->ainv);
  }
  // largest eigenvalue of M A on every smoothed level (power iteration; per
  // segment on the finest level of a packed plan)
  const int nseg = (plan->seg && plan->seg->nseg > 0) ? plan->seg->nseg : 0;
  if (nseg > mg->segn_n) {
    BT_CHECK(dalloc_n(mg, &mg->segn, 2 * (size_t)nseg));
    mg->segn_n = nseg;
  }
  MgDegrees dg{};
  dg.nlev = L;
  for (int l = 0; l < L; ++l) {
    MgLevel &c = mg->lv[l];
    dg.deg[l] = c.deg;
    const bool smoothed = l + 1 < L || (!mg->dense && !mg->coarse_blockdiag);
    if (!smoothed) continue;
    const int64_t n = (int64_t)c.bs * c.n;
    float *x = c.x, *y = c.x2;
    BT_LAUNCH(ctx, k_mg_hash_fill, grid_n(ctx, n), 256, 0, n, x, 0x9e3779b9u + 7919u * (unsigned)l);
    for (int it = 0; it < kPowerIters; ++it) {
      if (l == 0) {
        BT_CHECK(resid0(ctx, plan, values, nullptr, x, c.r, nullptr));
        if (sm.gl) {
          BT_CHECK(fac_lower(ctx, plan, sm, c.r, c.d, nullptr));
          BT_CHECK(fac_upper(ctx, plan, sm, c.d, nullptr, y, nullptr, nullptr, nullptr, nullptr));
        } else {
          BT_LAUNCH_PDL(ctx, k_mg0_bj, grid_n(ctx, plan->nV), 256, 0, plan->nV, sm.minv, c.r, y, (const float *)nullptr,
                    (const PcgState *)nullptr);
        }
      } else {
        BT_LAUNCH(ctx, k_mgc_MA<kGc>, grid_rows(ctx, c.n, kGc), 256, 0, c.n, c.rp, c.ci, c.val16, c.dinv, x, y);
      }
      if (it == kPowerIters - 2) BT_CHECK(sumsq_into(ctx, mg, n, y, mg->norms + 2 * l));
      if (it == kPowerIters - 1) BT_CHECK(sumsq_into(ctx, mg, n, y, mg->norms + 2 * l + 1));
      if (l == 0 && nseg > 0 && it >= kPowerIters - 2)
        BT_LAUNCH(ctx, k_mg_seg_sumsq, nseg, 256, 0, plan->seg->voff, y,
                  mg->segn + (it == kPowerIters - 1 ? nseg : 0));
      std::swap(x, y);
    }
    if (l == 0 && nseg > 0)
      BT_LAUNCH(ctx, k_mg_seg_lmax, 1, 32, 0, nseg, (const double *)mg->segn, (const double *)(mg->segn + nseg),
                mg->norms);
  }
  BT_LAUNCH(ctx, k_mg_coef, 1, 32, 0, dg, mg->norms, mg->coef);
  return BARTELS_OK;
}

int mg_enqueue_update(bartels_ctx ctx, bartels_mesh_plan plan, const MgSmoother &sm, const float *pa,
                      const float *pb, const float *ap, float *x, float *r, double *part, PcgState *st) {
  MgHierarchy *mg = plan->mg;
  BT_LAUNCH_PDL(ctx, k_mg0_update, grid_n(ctx, plan->nV), 256, 0, plan->nV, pa, pb, ap, x, r, sm.minv, mg->lv[0].x,
            (const float *)mg->coef, part, st);
  return BARTELS_OK;
}

int mg_enqueue_apply(bartels_ctx ctx, bartels_mesh_plan plan, const float *values, const MgSmoother &sm,
                     const float *r, float *z, float *y, double *part, PcgState *st, bool pre_done) {
  MgHierarchy *mg = plan->mg;
  MgLevel &l0 = mg->lv[0];
  const float *c0 = mg->coef;
  const int nV = plan->nV;
  if (sm.gl) {
    BT_CHECK(fac_lower(ctx, plan, sm, r, y, st));
    BT_CHECK(fac_upper(ctx, plan, sm, y, nullptr, l0.x, c0, nullptr, nullptr, st));
  } else if (!pre_done) {
    BT_LAUNCH_PDL(ctx, k_mg0_bj, grid_n(ctx, nV), 256, 0, nV, sm.minv, r, l0.x, c0, st);
  }
  BT_CHECK(resid0(ctx, plan, values, r, l0.x, l0.r, st));
  bool first_done = false;
  BT_CHECK(restrict_into<3>(ctx, mg, l0, l0.r, 1, st, &first_done));
  BT_CHECK(enqueue_coarse(ctx, mg, 1, first_done, st));
  BT_LAUNCH_PDL(ctx, k_mg_prolong<3>, grid_n(ctx, nV), 256, 0, nV, l0.agg, l0.Q, level_result(mg, 1), l0.x, st);
  if (sm.gl) {
    BT_CHECK(resid0(ctx, plan, values, r, l0.x, l0.r, st));
    BT_CHECK(fac_lower(ctx, plan, sm, l0.r, y, st));
    BT_CHECK(fac_upper(ctx, plan, sm, y, l0.x, z, c0, r, part, st));
  } else {
    using B16 = __nv_bfloat16;
    if (mg->a16) {
      const int G = plan_lanes_tri(ctx, plan);
      const int g = grid_rows(ctx, nV, G);
      BT_MG_G(G, BT_LAUNCH_PDL(ctx, (k_mg0_post_bj<GL, B16>), g, 256, 0, nV, plan->brp, plan->bcol,
                               (const B16 *)mg->a16, (const int *)mg->a16_off, sm.minv, r, l0.x, z, plan->pinned, c0,
                               part, st));
    } else {
      const int G = plan_lanes_spmv(ctx, plan);
      const int g = grid_rows(ctx, nV, G);
      BT_MG_G(G, BT_LAUNCH_PDL(ctx, (k_mg0_post_bj<GL, float>), g, 256, 0, nV, plan->brp, plan->bcol, values,
                               (const int *)nullptr, sm.minv, r, l0.x, z, plan->pinned, c0, part, st));
    }
  }
  return BARTELS_OK;
}

int mg_apply_once(bartels_ctx ctx, bartels_mesh_plan plan, const float *values, const MgSmoother &sm, const float *r,
                  float *z) {
  MgHierarchy *mg = plan->mg;
  if (!mg->st_once) {
    BT_CHECK(dalloc_n(mg, &mg->st_once, 1));
    BT_CUDA(cudaMemsetAsync(mg->st_once, 0, sizeof(PcgState), ctx->stream));
  }
  BT_CHECK(mg_enqueue_apply(ctx, plan, values, sm, r, z, mg->lv[0].d, mg->part, mg->st_once, false));
  BT_CUDA(cudaStreamSynchronize(ctx->stream));
  return BARTELS_OK;
}

}  // namespace bartels
