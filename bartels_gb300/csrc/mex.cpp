// MATLAB-gateway facade (include/bartels_mex.h): the argument conventions of the
// reference's matlab/<routine>.cpp gateways on top of the C ABI. Host code only.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <list>
#include <mutex>
#include <string>
#include <vector>

#include "bartels_gpu.h"
#include "bartels_mex.h"

namespace bartels {
int fail(int status, const std::string &msg);
}

namespace {

using bartels::fail;

enum Family { TET, TRI2, TRI3, ANY };
enum Op { DPHI, MASS, FIXED, Q, DQ, DQ2, LAW_DPSI, LAW_D2PSI };

struct Routine {
  const char *name;
  Family fam;
  Op op;
  int model;   // BARTELS_* law, -1 if none
  int nargs;   // arguments the gateway reads
  bool psd;    // gateway applies simple_psd_fix(1e-3) when given one more argument
};

#define TET_MODEL(m, M)                                           \
  {"linear_tetmesh_" #m "_q", TET, Q, M, 6, false},               \
  {"linear_tetmesh_" #m "_dq", TET, DQ, M, 6, false},             \
  {"linear_tetmesh_" #m "_dq2", TET, DQ2, M, 6, true}
#define TRI_MODEL(m, M)                                           \
  {"linear_tri2dmesh_" #m "_q", TRI2, Q, M, 6, false},            \
  {"linear_tri2dmesh_" #m "_dq", TRI2, DQ, M, 6, false},          \
  {"linear_tri2dmesh_" #m "_dq2", TRI2, DQ2, M, 6, true}

// One row per gateway of the reference's matlab/ directory on this path
// (matlab/linear_tetmesh_*.cpp, matlab/linear_tri2dmesh_*.cpp,
// matlab/linear_tri3dmesh_{dphi_dX,stvk_dq2}.cpp,
// matlab/fixed_point_constraint_matrix.cpp).
const Routine kRoutines[] = {
    {"linear_tetmesh_dphi_dX", TET, DPHI, -1, 2, false},
    {"linear_tetmesh_mass_matrix", TET, MASS, -1, 4, false},
    {"fixed_point_constraint_matrix", ANY, FIXED, -1, 2, false},
    TET_MODEL(neohookean, BARTELS_NEOHOOKEAN),
    TET_MODEL(stvk, BARTELS_STVK),
    TET_MODEL(corotational, BARTELS_COROTATIONAL),
    TET_MODEL(arap, BARTELS_ARAP),
    {"linear_tetmesh_linear_elasticity_dq2", TET, DQ2, BARTELS_LINEAR_ELASTICITY, 6, false},
    {"linear_tri2dmesh_dphi_dX", TRI2, DPHI, -1, 2, false},
    {"linear_tri2dmesh_mass_matrix", TRI2, MASS, -1, 4, false},
    TRI_MODEL(neohookean, BARTELS_NEOHOOKEAN),
    TRI_MODEL(stvk, BARTELS_STVK),
    TRI_MODEL(corotational, BARTELS_COROTATIONAL),
    TRI_MODEL(arap, BARTELS_ARAP),
    {"linear_tri2dmesh_linear_elasticity_dq2", TRI2, DQ2, BARTELS_LINEAR_ELASTICITY, 6, false},
    {"linear_tri3dmesh_dphi_dX", TRI3, DPHI, -1, 2, false},
    {"linear_tri3dmesh_stvk_dq2", TRI3, DQ2, BARTELS_STVK, 9, true},
    // matlab/dpsi_neohookean_dF.cpp, matlab/d2psi_neohookean_dF2.cpp, matlab/d2psi_stvk_dF2.cpp:
    // (E, F, params), one row of F and params per element of E
    {"dpsi_neohookean_dF", ANY, LAW_DPSI, BARTELS_NEOHOOKEAN, 3, false},
    {"d2psi_neohookean_dF2", ANY, LAW_D2PSI, BARTELS_NEOHOOKEAN, 3, false},
    {"d2psi_stvk_dF2", ANY, LAW_D2PSI, BARTELS_STVK, 3, false},
};
#undef TET_MODEL
#undef TRI_MODEL
constexpr int kNumRoutines = (int)(sizeof(kRoutines) / sizeof(kRoutines[0]));
constexpr double kGatewayPsdTol = 1e-3;  // matlab/linear_tetmesh_neohookean_dq2.cpp:40

int64_t numel(const bartels_mx &a) { return a.m * a.n; }

int check_shape(const bartels_mx &a, const char *what, int64_t m, int64_t n) {
  if (!a.pr && numel(a) > 0) return fail(BARTELS_E_INVALID_ARG, std::string(what) + ": no data");
  if ((m >= 0 && a.m != m) || (n >= 0 && a.n != n))
    return fail(BARTELS_E_INVALID_ARG, std::string(what) + ": expected " + (m >= 0 ? std::to_string(m) : "any") +
                                           " x " + (n >= 0 ? std::to_string(n) : "any") + ", got " +
                                           std::to_string(a.m) + " x " + std::to_string(a.n));
  return BARTELS_OK;
}

int check_numel(const bartels_mx &a, const char *what, int64_t count) {
  if (numel(a) != count || (count > 0 && !a.pr))
    return fail(BARTELS_E_INVALID_ARG, std::string(what) + ": expected " + std::to_string(count) + " entries, got " +
                                           std::to_string(numel(a)));
  return BARTELS_OK;
}

// 1-based MATLAB indices (doubles) -> 0-based ints; integral and in [1, limit].
int to_index(const bartels_mx &a, const char *what, int64_t limit, std::vector<int> &out) {
  out.resize((size_t)numel(a));
  for (size_t i = 0; i < out.size(); ++i) {
    const double v = a.pr[i];
    if (!(v >= 1.0 && v <= (double)limit) || v != std::floor(v))
      return fail(BARTELS_E_INVALID_ARG, std::string(what) + ": entry " + std::to_string(i) +
                                             " is not a 1-based index in [1, " + std::to_string(limit) + "]");
    out[i] = (int)v - 1;
  }
  return BARTELS_OK;
}

// Cached mesh plan with its CSR pattern and the transpose permutation that
// turns CSR values into MATLAB's compressed columns.
struct Entry {
  Family fam;
  std::vector<double> V;  // tets: rest positions the plan was built from
  std::vector<int> E;     // 0-based, column-major
  int nV = 0, nT = 0;
  bartels_mesh_plan tet = nullptr;
  bartels_tri_plan tri = nullptr;
  int n = 0;
  std::vector<int> rp, ci;
  std::vector<int64_t> tperm;
};

struct State {
  std::mutex mu;
  bartels_ctx ctx = nullptr;
  std::list<Entry> plans;  // most recently used first
};
State &state() {
  static State s;
  return s;
}
constexpr size_t kMaxPlans = 4;

void free_entry(Entry &e) {
  if (e.tet) bartels_plan_destroy(e.tet);
  if (e.tri) bartels_tri_plan_destroy(e.tri);
  e.tet = nullptr;
  e.tri = nullptr;
}

int get_ctx(bartels_ctx *out) {
  State &s = state();
  if (!s.ctx) {
    const int st = bartels_ctx_create(0, &s.ctx);
    if (st != BARTELS_OK) {
      s.ctx = nullptr;
      return st;
    }
  }
  *out = s.ctx;
  return BARTELS_OK;
}

// For a structurally symmetric CSR pattern, tperm[p] is the position of the
// entry transposed to p; MATLAB's column j is then the CSR row j with values
// vals[tperm[p]], i.e. H(row, j) for every stored row.
int build_transpose(Entry &e) {
  const int64_t nnz = e.rp[e.n];
  e.tperm.resize((size_t)nnz);
  for (int r = 0; r < e.n; ++r)
    for (int p = e.rp[r]; p < e.rp[r + 1]; ++p) {
      const int c = e.ci[p];
      const int *b = e.ci.data() + e.rp[c], *end = e.ci.data() + e.rp[c + 1];
      const int *f = std::lower_bound(b, end, r);
      if (f == end || *f != r) return fail(BARTELS_E_DEVICE, "CSR pattern is not structurally symmetric");
      e.tperm[p] = f - e.ci.data();
    }
  return BARTELS_OK;
}

int get_plan(Family fam, int nV, const bartels_mx &Vm, int nT, const std::vector<int> &E, Entry **out) {
  State &s = state();
  const bool keyV = fam == TET;
  for (auto it = s.plans.begin(); it != s.plans.end(); ++it) {
    if (it->fam != fam || it->nV != nV || it->nT != nT || it->E != E) continue;
    if (keyV && std::memcmp(it->V.data(), Vm.pr, sizeof(double) * it->V.size()) != 0) continue;
    s.plans.splice(s.plans.begin(), s.plans, it);
    *out = &s.plans.front();
    return BARTELS_OK;
  }
  bartels_ctx ctx;
  int st = get_ctx(&ctx);
  if (st != BARTELS_OK) return st;
  Entry e;
  e.fam = fam;
  e.nV = nV;
  e.nT = nT;
  e.E = E;
  int64_t nnz = 0;
  if (fam == TET) {
    e.V.assign(Vm.pr, Vm.pr + 3 * (size_t)nV);
    st = bartels_plan_create(ctx, nV, Vm.pr, nT, E.data(), &e.tet);
    if (st == BARTELS_OK) st = bartels_plan_csr_size(e.tet, &e.n, &nnz);
    if (st == BARTELS_OK) {
      e.rp.resize((size_t)e.n + 1);
      e.ci.resize((size_t)nnz);
      st = bartels_plan_csr_pattern(e.tet, e.rp.data(), e.ci.data());
    }
  } else {
    st = bartels_tri_plan_create(ctx, nV, nT, E.data(), fam == TRI2 ? 2 : 3, &e.tri);
    if (st == BARTELS_OK) st = bartels_tri_plan_csr_size(e.tri, &e.n, &nnz);
    if (st == BARTELS_OK) {
      e.rp.resize((size_t)e.n + 1);
      e.ci.resize((size_t)nnz);
      st = bartels_tri_plan_csr_pattern(e.tri, e.rp.data(), e.ci.data());
    }
  }
  if (st == BARTELS_OK) st = build_transpose(e);
  if (st != BARTELS_OK) {
    free_entry(e);
    return st;
  }
  s.plans.push_front(std::move(e));
  while (s.plans.size() > kMaxPlans) {
    free_entry(s.plans.back());
    s.plans.pop_back();
  }
  *out = &s.plans.front();
  return BARTELS_OK;
}

int alloc_dense(bartels_mx_alloc alloc, void *user, int64_t m, int64_t n, double **pr) {
  *pr = nullptr;
  if (alloc(user, m, n, -1, pr, nullptr, nullptr) != 0 || (m * n > 0 && !*pr))
    return fail(BARTELS_E_INVALID_ARG, "output allocation failed");
  return BARTELS_OK;
}

// CSR values of a plan's symmetric pattern -> MATLAB sparse n x n.
int emit_sparse(const Entry &e, const std::vector<double> &vals, bartels_mx_alloc alloc, void *user) {
  const int64_t nnz = e.rp[e.n];
  double *pr = nullptr;
  uint64_t *ir = nullptr, *jc = nullptr;
  if (alloc(user, e.n, e.n, nnz, &pr, &ir, &jc) != 0 || !jc || (nnz > 0 && (!pr || !ir)))
    return fail(BARTELS_E_INVALID_ARG, "output allocation failed");
  for (int j = 0; j <= e.n; ++j) jc[j] = (uint64_t)e.rp[j];
  for (int64_t p = 0; p < nnz; ++p) {
    ir[p] = (uint64_t)e.ci[p];
    pr[p] = vals[(size_t)e.tperm[p]];
  }
  return BARTELS_OK;
}

// params: nT x 2 as the kernels read them; ARAP reads only column 0 and
// accepts nT x 1 (src/psi_arap_S.cpp:8 uses params(0)).
int params2(const bartels_mx &a, int nT, int model, std::vector<double> &out) {
  const int64_t need = model == BARTELS_ARAP ? 1 : 2;
  if (a.m != nT || a.n < need || !a.pr)
    return fail(BARTELS_E_INVALID_ARG, "params: expected " + std::to_string(nT) + " x " + std::to_string(need) +
                                           " (or more columns), got " + std::to_string(a.m) + " x " +
                                           std::to_string(a.n));
  out.assign(2 * (size_t)nT, 0.0);
  std::memcpy(out.data(), a.pr, sizeof(double) * (size_t)nT * (size_t)std::min<int64_t>(a.n, 2));
  return BARTELS_OK;
}

int fixed_point(int nrhs, const bartels_mx *prhs, bartels_mx_alloc alloc, void *user) {
  const bartels_mx &V = prhs[0];
  if (V.n <= 0 || V.m < 0 || V.m > INT32_MAX / 3) return fail(BARTELS_E_INVALID_ARG, "V: bad size");
  const int nV = (int)V.m, dim = (int)V.n;
  std::vector<int> fixed;
  int st = to_index(prhs[1], "fixed", nV, fixed);
  if (st != BARTELS_OK) return st;
  int rows = 0;
  st = bartels_fixed_point_constraint_matrix(nV, dim, fixed.data(), (int)fixed.size(), &rows, nullptr, nullptr,
                                             nullptr);
  if (st != BARTELS_OK) return st;
  // One 1 per row, at the free DOF's column: column c holds row r iff DOF c is
  // the r-th free DOF, so the columns are the rows' transpose in order.
  std::vector<int> rp((size_t)rows + 1), ci((size_t)rows);
  st = bartels_fixed_point_constraint_matrix(nV, dim, fixed.data(), (int)fixed.size(), &rows, rp.data(), ci.data(),
                                             nullptr);
  if (st != BARTELS_OK) return st;
  const int64_t ncol = (int64_t)dim * nV;
  double *pr = nullptr;
  uint64_t *ir = nullptr, *jc = nullptr;
  if (alloc(user, rows, ncol, rows, &pr, &ir, &jc) != 0 || !jc || (rows > 0 && (!pr || !ir)))
    return fail(BARTELS_E_INVALID_ARG, "output allocation failed");
  int r = 0;
  for (int64_t c = 0; c < ncol; ++c) {
    jc[c] = (uint64_t)r;
    if (r < rows && ci[(size_t)r] == c) {
      ir[r] = (uint64_t)r;
      pr[r] = 1.0;
      ++r;
    }
  }
  jc[ncol] = (uint64_t)r;
  (void)nrhs;
  return BARTELS_OK;
}

// The gateways loop over the rows of E (only its row count is used) and hand
// back dpsi as one 9 nT vector (element after element) and d2psi as the
// 9 nT x 9 nT block-diagonal sparse matrix with every block entry stored.
int pointwise(const Routine &R, const bartels_mx *prhs, bartels_mx_alloc alloc, void *user) {
  const int64_t nT = prhs[0].m;
  if (nT < 0 || nT > INT32_MAX / 81) return fail(BARTELS_E_UNSUPPORTED, "E: too many elements");
  int st = check_shape(prhs[1], "F", nT, 9);
  if (st != BARTELS_OK) return st;
  std::vector<double> pbuf;
  if ((st = params2(prhs[2], (int)nT, R.model, pbuf)) != BARTELS_OK) return st;
  bartels_ctx ctx;
  if ((st = get_ctx(&ctx)) != BARTELS_OK) return st;
  const size_t n = (size_t)nT;
  if (R.op == LAW_DPSI) {
    std::vector<double> d(9 * n);
    if (n && (st = bartels_pointwise_laws(ctx, R.model, (int)nT, prhs[1].pr, pbuf.data(), nullptr, d.data(),
                                          nullptr)) != BARTELS_OK)
      return st;
    double *out;
    if ((st = alloc_dense(alloc, user, 9 * nT, 1, &out)) != BARTELS_OK) return st;
    for (size_t t = 0; t < n; ++t)
      for (int r = 0; r < 9; ++r) out[9 * t + r] = d[t + n * r];
    return BARTELS_OK;
  }
  std::vector<double> H(81 * n);
  if (n && (st = bartels_pointwise_laws(ctx, R.model, (int)nT, prhs[1].pr, pbuf.data(), nullptr, nullptr,
                                        H.data())) != BARTELS_OK)
    return st;
  double *pr = nullptr;
  uint64_t *ir = nullptr, *jc = nullptr;
  const int64_t nnz = 81 * nT;
  if (alloc(user, 9 * nT, 9 * nT, nnz, &pr, &ir, &jc) != 0 || !jc || (nnz > 0 && (!pr || !ir)))
    return fail(BARTELS_E_INVALID_ARG, "output allocation failed");
  for (size_t t = 0; t < n; ++t)
    for (int c = 0; c < 9; ++c) {
      jc[9 * t + c] = 81 * t + 9 * c;
      for (int r = 0; r < 9; ++r) {
        ir[81 * t + 9 * c + r] = 9 * t + r;
        pr[81 * t + 9 * c + r] = H[81 * t + r + 9 * c];
      }
    }
  jc[9 * n] = (uint64_t)nnz;
  return BARTELS_OK;
}

int run(const Routine &R, int nrhs, const bartels_mx *prhs, bartels_mx_alloc alloc, void *user) {
  if (R.op == FIXED) return fixed_point(nrhs, prhs, alloc, user);
  if (R.op == LAW_DPSI || R.op == LAW_D2PSI) return pointwise(R, prhs, alloc, user);
  // ---- validation (host only, before any device work)
  const int vdim = R.fam == TRI2 ? 2 : 3;                 // columns of V
  const int nodes = R.fam == TET ? 4 : 3;                  // columns of E
  const int dofs = R.fam == TRI2 ? 2 : 3;                  // DOFs per vertex
  const int ndphi = R.fam == TET ? 12 : (R.fam == TRI2 ? 6 : 9);
  int st = check_shape(prhs[0], "V", -1, vdim);
  if (st != BARTELS_OK) return st;
  st = check_shape(prhs[1], "E", -1, nodes);
  if (st != BARTELS_OK) return st;
  if (prhs[0].m > INT32_MAX / 3 || prhs[1].m > INT32_MAX / 12) return fail(BARTELS_E_UNSUPPORTED, "mesh too large");
  const int nV = (int)prhs[0].m, nT = (int)prhs[1].m;
  std::vector<int> E;
  st = to_index(prhs[1], "E", nV, E);
  if (st != BARTELS_OK) return st;

  const bartels_mx *q = nullptr, *dphi = nullptr, *vol = nullptr, *par = nullptr, *dens = nullptr;
  const bartels_mx *Nr = nullptr, *nd = nullptr, *dndq = nullptr;
  std::vector<double> pbuf;
  if (R.op == MASS) {
    dens = &prhs[2];
    vol = &prhs[3];
    if ((st = check_numel(*dens, "densities", nT)) != BARTELS_OK) return st;
    if ((st = check_numel(*vol, R.fam == TET ? "volumes" : "areas", nT)) != BARTELS_OK) return st;
  } else if (R.op != DPHI) {
    q = &prhs[2];
    dphi = &prhs[3];
    if ((st = check_numel(*q, "q", (int64_t)dofs * nV)) != BARTELS_OK) return st;
    if ((st = check_shape(*dphi, "dphidX", nT, ndphi)) != BARTELS_OK) return st;
    int k = 4;
    if (R.fam == TRI3) {
      Nr = &prhs[4];
      nd = &prhs[5];
      dndq = &prhs[6];
      if ((st = check_shape(*Nr, "N", nT, 3)) != BARTELS_OK) return st;
      if ((st = check_shape(*nd, "n", nT, 3)) != BARTELS_OK) return st;
      if ((st = check_shape(*dndq, "dndq", nT, 27)) != BARTELS_OK) return st;
      k = 7;
    }
    vol = &prhs[k];
    par = &prhs[k + 1];
    if ((st = check_numel(*vol, R.fam == TET ? "volumes" : "areas", nT)) != BARTELS_OK) return st;
    if ((st = params2(*par, nT, R.model, pbuf)) != BARTELS_OK) return st;
  }
  const int psd = (R.psd && nrhs > R.nargs) ? BARTELS_PSD_SIMPLE_FIX : BARTELS_PSD_NONE;

  // ---- device work
  bartels_ctx ctx;
  if ((st = get_ctx(&ctx)) != BARTELS_OK) return st;
  if (R.op == DPHI) {
    double *out;
    if ((st = alloc_dense(alloc, user, nT, ndphi, &out)) != BARTELS_OK) return st;
    if (nT == 0) return BARTELS_OK;
    if (R.fam == TET) return bartels_tetmesh_dphi_dX(ctx, nV, prhs[0].pr, nT, E.data(), out);
    if (R.fam == TRI2) return bartels_tri2dmesh_dphi_dX(ctx, nV, prhs[0].pr, nT, E.data(), out, nullptr);
    return bartels_tri3dmesh_dphi_dX(ctx, nV, prhs[0].pr, nT, E.data(), out, nullptr);
  }
  if (nT == 0) return fail(BARTELS_E_INVALID_ARG, "E: empty mesh");
  Entry *e = nullptr;
  if ((st = get_plan(R.fam, nV, prhs[0], nT, E, &e)) != BARTELS_OK) return st;
  const int64_t nnz = e->rp[e->n];
  if (R.op == MASS) {
    std::vector<double> vals((size_t)nnz);
    st = R.fam == TET ? bartels_tetmesh_mass_matrix(ctx, e->tet, dens->pr, vol->pr, vals.data())
                      : bartels_tri2dmesh_mass_matrix(ctx, e->tri, dens->pr, vol->pr, vals.data());
    if (st != BARTELS_OK) return st;
    return emit_sparse(*e, vals, alloc, user);
  }
  if (R.op == Q) {
    double energy = 0.0;
    st = R.fam == TET ? bartels_tetmesh_q(ctx, e->tet, R.model, q->pr, dphi->pr, vol->pr, pbuf.data(), &energy)
                      : bartels_tri2dmesh_q(ctx, e->tri, R.model, q->pr, dphi->pr, vol->pr, pbuf.data(), &energy);
    if (st != BARTELS_OK) return st;
    double *out;
    if ((st = alloc_dense(alloc, user, 1, 1, &out)) != BARTELS_OK) return st;
    *out = energy;
    return BARTELS_OK;
  }
  if (R.op == DQ) {
    double *out;
    if ((st = alloc_dense(alloc, user, (int64_t)dofs * nV, 1, &out)) != BARTELS_OK) return st;
    return R.fam == TET ? bartels_tetmesh_dq(ctx, e->tet, R.model, q->pr, dphi->pr, vol->pr, pbuf.data(), out)
                        : bartels_tri2dmesh_dq(ctx, e->tri, R.model, q->pr, dphi->pr, vol->pr, pbuf.data(), out);
  }
  std::vector<double> vals((size_t)nnz);
  if (R.fam == TET)
    st = bartels_tetmesh_dq2(ctx, e->tet, R.model, q->pr, dphi->pr, vol->pr, pbuf.data(), psd, kGatewayPsdTol, 0,
                             vals.data());
  else if (R.fam == TRI2)
    st = bartels_tri2dmesh_dq2(ctx, e->tri, R.model, q->pr, dphi->pr, vol->pr, pbuf.data(), psd, kGatewayPsdTol,
                               vals.data());
  else
    st = bartels_tri3dmesh_stvk_dq2(ctx, e->tri, q->pr, dphi->pr, Nr->pr, nd->pr, dndq->pr, vol->pr, pbuf.data(),
                                    psd, kGatewayPsdTol, vals.data());
  if (st != BARTELS_OK) return st;
  return emit_sparse(*e, vals, alloc, user);
}

}  // namespace

extern "C" {

int bartels_mex_call(const char *routine, int nrhs, const bartels_mx *prhs, bartels_mx_alloc alloc, void *user) {
  if (!routine || !alloc || nrhs < 0 || (nrhs > 0 && !prhs)) return fail(BARTELS_E_INVALID_ARG, "bad arguments");
  const Routine *R = nullptr;
  for (const Routine &r : kRoutines)
    if (std::strcmp(r.name, routine) == 0) R = &r;
  if (!R) return fail(BARTELS_E_INVALID_ARG, std::string("unknown routine ") + routine);
  if (nrhs < R->nargs)
    return fail(BARTELS_E_INVALID_ARG, std::string(routine) + " takes " + std::to_string(R->nargs) +
                                           " arguments, got " + std::to_string(nrhs));
  std::lock_guard<std::mutex> lock(state().mu);
  return run(*R, nrhs, prhs, alloc, user);
}

int bartels_mex_routine_count(void) { return kNumRoutines; }

const char *bartels_mex_routine_name(int i) { return (i >= 0 && i < kNumRoutines) ? kRoutines[i].name : nullptr; }

void bartels_mex_release(void) {
  State &s = state();
  std::lock_guard<std::mutex> lock(s.mu);
  for (Entry &e : s.plans) free_entry(e);
  s.plans.clear();
  if (s.ctx) bartels_ctx_destroy(s.ctx);
  s.ctx = nullptr;
}

}  // extern "C"
