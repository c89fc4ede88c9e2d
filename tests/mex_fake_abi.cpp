// Host-only test of the MATLAB-gateway facade (bartels_gb300/csrc/mex.cpp)
// linked against a stand-in of the C ABI that returns recognisable values:
// Hessian entry (i, j) = 100000 i + j + 0.5, deliberately unsymmetric, so the
// compressed columns must carry H(i, j) and not H(j, i); dphidX entry (t, c) =
// 100 t + c; dpsi(t, r) = 10 t + r; d2psi block t (r, c) = 1000 t + 10 r + c;
// energy = sum of q (q reaches the ABI unshifted). Also the plan cache (hits,
// misses on a changed V or E, eviction) and 1-based index conversion.
// Prints "mex facade ok" and returns 0 on success.
#include <cstdio>
#include <cstring>
#include <set>
#include <string>
#include <vector>

#include "bartels_gpu.h"
#include "bartels_mex.h"

namespace bartels {
static std::string g_err;
int fail(int status, const std::string &msg) {
  g_err = msg;
  return status;
}
}  // namespace bartels

// ------------------------------------------------------------- stand-in ABI --
static int ctx_created = 0, plans_created = 0, plans_destroyed = 0;
static int ctx_storage;

struct FakePlan {
  int nV = 0, nT = 0, dim = 3, nodes = 4;
  std::vector<int> E, rp, ci;
};
struct bartels_mesh_plan_s : FakePlan {};
struct bartels_tri_plan_s : FakePlan {};

static void build_pattern(FakePlan &p) {
  std::vector<std::set<int>> nb(p.nV);
  for (int t = 0; t < p.nT; ++t)
    for (int a = 0; a < p.nodes; ++a)
      for (int b = 0; b < p.nodes; ++b) nb[p.E[t + p.nT * a]].insert(p.E[t + p.nT * b]);
  p.rp.assign(1, 0);
  p.ci.clear();
  for (int v = 0; v < p.nV; ++v)
    for (int k = 0; k < p.dim; ++k) {
      for (int j : nb[v])
        for (int l = 0; l < p.dim; ++l) p.ci.push_back(p.dim * j + l);
      p.rp.push_back((int)p.ci.size());
    }
}

static void fill_unsymmetric(const FakePlan &p, double *vals) {
  for (int r = 0; r + 1 < (int)p.rp.size(); ++r)
    for (int k = p.rp[r]; k < p.rp[r + 1]; ++k) vals[k] = 100000.0 * r + p.ci[k] + 0.5;
}

extern "C" {
int bartels_ctx_create(int, bartels_ctx *out) {
  ++ctx_created;
  *out = reinterpret_cast<bartels_ctx>(&ctx_storage);
  return BARTELS_OK;
}
int bartels_ctx_destroy(bartels_ctx) { return BARTELS_OK; }
int bartels_plan_create(bartels_ctx, int nV, const double *, int nT, const int *E, bartels_mesh_plan *out) {
  auto *p = new bartels_mesh_plan_s;
  p->nV = nV;
  p->nT = nT;
  p->E.assign(E, E + 4 * (size_t)nT);
  build_pattern(*p);
  ++plans_created;
  *out = p;
  return BARTELS_OK;
}
int bartels_plan_destroy(bartels_mesh_plan p) {
  ++plans_destroyed;
  delete p;
  return BARTELS_OK;
}
int bartels_plan_csr_size(bartels_mesh_plan p, int *n, int64_t *nnz) {
  *n = (int)p->rp.size() - 1;
  *nnz = (int64_t)p->ci.size();
  return BARTELS_OK;
}
int bartels_plan_csr_pattern(bartels_mesh_plan p, int *rp, int *ci) {
  std::memcpy(rp, p->rp.data(), sizeof(int) * p->rp.size());
  std::memcpy(ci, p->ci.data(), sizeof(int) * p->ci.size());
  return BARTELS_OK;
}
int bartels_tri_plan_create(bartels_ctx, int nV, int nT, const int *E, int dim, bartels_tri_plan *out) {
  auto *p = new bartels_tri_plan_s;
  p->nV = nV;
  p->nT = nT;
  p->dim = dim;
  p->nodes = 3;
  p->E.assign(E, E + 3 * (size_t)nT);
  build_pattern(*p);
  ++plans_created;
  *out = p;
  return BARTELS_OK;
}
void bartels_tri_plan_destroy(bartels_tri_plan p) {
  ++plans_destroyed;
  delete p;
}
int bartels_tri_plan_csr_size(bartels_tri_plan p, int *n, int64_t *nnz) {
  *n = (int)p->rp.size() - 1;
  *nnz = (int64_t)p->ci.size();
  return BARTELS_OK;
}
int bartels_tri_plan_csr_pattern(bartels_tri_plan p, int *rp, int *ci) {
  std::memcpy(rp, p->rp.data(), sizeof(int) * p->rp.size());
  std::memcpy(ci, p->ci.data(), sizeof(int) * p->ci.size());
  return BARTELS_OK;
}
static int fill_dphi(int nT, int ncols, double *out) {
  for (int t = 0; t < nT; ++t)
    for (int c = 0; c < ncols; ++c) out[t + (size_t)nT * c] = 100.0 * t + c;
  return BARTELS_OK;
}
int bartels_tetmesh_dphi_dX(bartels_ctx, int, const double *, int nT, const int *, double *d) {
  return fill_dphi(nT, 12, d);
}
int bartels_tri2dmesh_dphi_dX(bartels_ctx, int, const double *, int nT, const int *, double *d, double *) {
  return fill_dphi(nT, 6, d);
}
int bartels_tri3dmesh_dphi_dX(bartels_ctx, int, const double *, int nT, const int *, double *d, double *) {
  return fill_dphi(nT, 9, d);
}
int bartels_tetmesh_q(bartels_ctx, bartels_mesh_plan p, int, const double *q, const double *, const double *,
                      const double *, double *e) {
  double s = 0;
  for (int i = 0; i < 3 * p->nV; ++i) s += q[i];
  *e = s;
  return BARTELS_OK;
}
int bartels_tetmesh_dq(bartels_ctx, bartels_mesh_plan p, int, const double *q, const double *, const double *,
                       const double *, double *g) {
  for (int i = 0; i < 3 * p->nV; ++i) g[i] = 2.0 * q[i];
  return BARTELS_OK;
}
int bartels_tetmesh_dq2(bartels_ctx, bartels_mesh_plan p, int, const double *, const double *, const double *,
                        const double *, int, double, int, double *vals) {
  fill_unsymmetric(*p, vals);
  return BARTELS_OK;
}
int bartels_tetmesh_mass_matrix(bartels_ctx, bartels_mesh_plan p, const double *, const double *, double *vals) {
  fill_unsymmetric(*p, vals);
  return BARTELS_OK;
}
int bartels_tri2dmesh_q(bartels_ctx, bartels_tri_plan p, int, const double *q, const double *, const double *,
                        const double *, double *e) {
  double s = 0;
  for (int i = 0; i < 2 * p->nV; ++i) s += q[i];
  *e = s;
  return BARTELS_OK;
}
int bartels_tri2dmesh_dq(bartels_ctx, bartels_tri_plan p, int, const double *q, const double *, const double *,
                         const double *, double *g) {
  for (int i = 0; i < 2 * p->nV; ++i) g[i] = 2.0 * q[i];
  return BARTELS_OK;
}
int bartels_tri2dmesh_dq2(bartels_ctx, bartels_tri_plan p, int, const double *, const double *, const double *,
                          const double *, int, double, double *vals) {
  fill_unsymmetric(*p, vals);
  return BARTELS_OK;
}
int bartels_tri2dmesh_mass_matrix(bartels_ctx, bartels_tri_plan p, const double *, const double *, double *vals) {
  fill_unsymmetric(*p, vals);
  return BARTELS_OK;
}
int bartels_tri3dmesh_stvk_dq2(bartels_ctx, bartels_tri_plan p, const double *, const double *, const double *,
                               const double *, const double *, const double *, const double *, int, double,
                               double *vals) {
  fill_unsymmetric(*p, vals);
  return BARTELS_OK;
}
int bartels_fixed_point_constraint_matrix(int nV, int dim, const int *fixed, int nfix, int *rows, int *rp, int *ci,
                                          double *vals) {
  *rows = dim * (nV - nfix);
  if (!rp) return BARTELS_OK;
  int r = 0, f = 0;
  rp[0] = 0;
  for (int v = 0; v < nV; ++v) {
    if (f < nfix && fixed[f] == v) {
      ++f;
      continue;
    }
    for (int k = 0; k < dim; ++k) {
      if (ci) ci[r] = dim * v + k;
      if (vals) vals[r] = 1.0;
      ++r;
      rp[r] = r;
    }
  }
  return BARTELS_OK;
}
int bartels_pointwise_laws(bartels_ctx, int, int n, const double *, const double *, double *psi, double *dpsi,
                           double *d2psi) {
  for (int t = 0; t < n; ++t) {
    if (psi) psi[t] = t;
    for (int r = 0; r < 9; ++r) {
      if (dpsi) dpsi[t + (size_t)n * r] = 10.0 * t + r;
      for (int c = 0; c < 9; ++c)
        if (d2psi) d2psi[81 * (size_t)t + r + 9 * c] = 1000.0 * t + 10.0 * r + c;
    }
  }
  return BARTELS_OK;
}
}  // extern "C"

// ------------------------------------------------------------------ driver --
struct Out {
  int64_t m = 0, n = 0, nnz = -1;
  std::vector<double> pr;
  std::vector<uint64_t> ir, jc;
};
static int alloc(void *u, int64_t m, int64_t n, int64_t nnz, double **pr, uint64_t **ir, uint64_t **jc) {
  Out *o = static_cast<Out *>(u);
  o->m = m;
  o->n = n;
  o->nnz = nnz;
  if (nnz < 0) {
    o->pr.assign((size_t)(m * n), 0.0);
    *pr = o->pr.data();
    return 0;
  }
  o->pr.assign((size_t)(nnz > 0 ? nnz : 1), 0.0);
  o->ir.assign((size_t)(nnz > 0 ? nnz : 1), 0);
  o->jc.assign((size_t)n + 1, 0);
  *pr = o->pr.data();
  *ir = o->ir.data();
  *jc = o->jc.data();
  return 0;
}

#define REQUIRE(c)                                                          \
  do {                                                                      \
    if (!(c)) {                                                             \
      std::fprintf(stderr, "check failed: %s (line %d)\n", #c, __LINE__); \
      return 1;                                                             \
    }                                                                       \
  } while (0)

// every stored (i, j) of a compressed-column result must hold 100000 i + j + 0.5
static bool columns_hold_h_ij(const Out &o) {
  if (o.nnz < 0 || (int64_t)o.jc.size() != o.n + 1) return false;
  for (int64_t j = 0; j < o.n; ++j)
    for (uint64_t k = o.jc[j]; k < o.jc[j + 1]; ++k) {
      if (k > o.jc[j] && o.ir[k] <= o.ir[k - 1]) return false;  // ascending rows
      if (o.pr[k] != 100000.0 * (double)o.ir[k] + (double)j + 0.5) return false;
    }
  return o.jc[o.n] == (uint64_t)o.nnz;
}

int main() {
  // two tets sharing the face (1, 2, 3): 5 vertices; E 1-based doubles, column-major
  std::vector<double> V = {0, 1, 0, 0, 1, 0, 0, 1, 0, -1, 0, 0, 1, 0, -1}, q(15);
  for (int i = 0; i < 15; ++i) q[i] = 1.0 + 0.25 * i;
  const double E1[8] = {1, 5, 2, 2, 3, 3, 4, 4};
  std::vector<double> dphi(24, 0.0), vol(2, 1.0), params(4, 1.0);
  bartels_mx in[9] = {{5, 3, V.data()}, {2, 4, E1}, {15, 1, q.data()}, {2, 12, dphi.data()}, {2, 1, vol.data()},
                      {2, 2, params.data()}};
  Out o;
  REQUIRE(bartels_mex_call("linear_tetmesh_neohookean_dq2", 6, in, alloc, &o) == BARTELS_OK);
  REQUIRE(o.m == 15 && o.n == 15 && columns_hold_h_ij(o));
  REQUIRE(plans_created == 1 && ctx_created == 1);
  // same mesh: cached; a changed V or E: a new plan
  REQUIRE(bartels_mex_call("linear_tetmesh_stvk_dq2", 7, in, alloc, &o) == BARTELS_OK && plans_created == 1);
  V[0] = 0.5;
  REQUIRE(bartels_mex_call("linear_tetmesh_stvk_dq2", 6, in, alloc, &o) == BARTELS_OK && plans_created == 2);
  const double E2[8] = {1, 5, 3, 2, 2, 3, 4, 4};
  in[1].pr = E2;
  REQUIRE(bartels_mex_call("linear_tetmesh_mass_matrix", 4,
                           std::vector<bartels_mx>{in[0], in[1], in[4], in[4]}.data(), alloc, &o) == BARTELS_OK);
  REQUIRE(plans_created == 3 && columns_hold_h_ij(o));
  in[1].pr = E1;
  // q reaches the ABI as given (no parse_rhs_index shift): energy = sum q
  REQUIRE(bartels_mex_call("linear_tetmesh_arap_q", 6, in, alloc, &o) == BARTELS_OK);
  double sq = 0;
  for (double v : q) sq += v;
  REQUIRE(o.nnz < 0 && o.m == 1 && o.n == 1 && o.pr[0] == sq);
  REQUIRE(bartels_mex_call("linear_tetmesh_corotational_dq", 6, in, alloc, &o) == BARTELS_OK);
  REQUIRE(o.m == 15 && o.n == 1 && o.pr[14] == 2.0 * q[14]);
  // dphidX comes back nT x 12 column-major
  REQUIRE(bartels_mex_call("linear_tetmesh_dphi_dX", 2, in, alloc, &o) == BARTELS_OK);
  REQUIRE(o.m == 2 && o.n == 12 && o.pr[1 + 2 * 11] == 100.0 + 11);
  // 1-based indices are checked: 0 and 6 are out of range, 2.5 is not integral
  for (double bad : {0.0, 6.0, 2.5}) {
    double Eb[8] = {1, 5, 2, 2, 3, 3, 4, 4};
    Eb[3] = bad;
    in[1].pr = Eb;
    REQUIRE(bartels_mex_call("linear_tetmesh_neohookean_q", 6, in, alloc, &o) == BARTELS_E_INVALID_ARG);
  }
  in[1].pr = E1;
  // planar triangles: 2 DOFs per vertex, pattern and H(i, j) as for tets
  std::vector<double> V2 = {0, 1, 0, 1, 0, 0, 1, 1}, q2(8, 0.5), d6(12, 0.0), a2(2, 0.5), p2(4, 1.0);
  const double T1[6] = {1, 2, 2, 4, 3, 3};
  bartels_mx tri[7] = {{4, 2, V2.data()}, {2, 3, T1}, {8, 1, q2.data()}, {2, 6, d6.data()}, {2, 1, a2.data()},
                       {2, 2, p2.data()}, {1, 1, a2.data()}};
  REQUIRE(bartels_mex_call("linear_tri2dmesh_corotational_dq2", 7, tri, alloc, &o) == BARTELS_OK);
  REQUIRE(o.m == 8 && o.n == 8 && columns_hold_h_ij(o));
  // pointwise laws: element-major dpsi, block-diagonal d2psi with block (r, c) at (9t + r, 9t + c)
  std::vector<double> F(27, 0.0), pl(6, 1.0), Ep(12, 1.0);
  bartels_mx pw[3] = {{3, 4, Ep.data()}, {3, 9, F.data()}, {3, 2, pl.data()}};
  REQUIRE(bartels_mex_call("dpsi_neohookean_dF", 3, pw, alloc, &o) == BARTELS_OK);
  REQUIRE(o.m == 27 && o.n == 1 && o.pr[9 * 2 + 4] == 24.0);
  REQUIRE(bartels_mex_call("d2psi_stvk_dF2", 3, pw, alloc, &o) == BARTELS_OK);
  REQUIRE(o.m == 27 && o.n == 27 && o.nnz == 243);
  for (int t = 0; t < 3; ++t)
    for (int c = 0; c < 9; ++c)
      for (int r = 0; r < 9; ++r) {
        const uint64_t k = o.jc[9 * t + c] + r;
        REQUIRE(o.ir[k] == (uint64_t)(9 * t + r) && o.pr[k] == 1000.0 * t + 10.0 * r + c);
      }
  // fixed_point_constraint_matrix: column c holds the row of free DOF c
  const double fixed[2] = {2, 4};
  bartels_mx fx[2] = {{5, 3, V.data()}, {2, 1, fixed}};
  REQUIRE(bartels_mex_call("fixed_point_constraint_matrix", 2, fx, alloc, &o) == BARTELS_OK);
  REQUIRE(o.m == 9 && o.n == 15 && o.nnz == 9 && o.jc[3] == 3 && o.jc[6] == 3 && o.ir[3] == 3);
  // eviction: the four most recent meshes stay cached, older plans are destroyed
  const int before = plans_destroyed;
  for (int s = 0; s < 5; ++s) {
    V[1] = 10.0 + s;
    REQUIRE(bartels_mex_call("linear_tetmesh_neohookean_dq", 6, in, alloc, &o) == BARTELS_OK);
  }
  REQUIRE(plans_destroyed > before);
  bartels_mex_release();
  std::printf("mex facade ok: %d plans created, %d destroyed\n", plans_created, plans_destroyed);
  return 0;
}
