// bartels_sim.hpp -- header-only C++ layer with the reference's names and
// argument order (namespace sim, include/linear_tetmesh_*.h of Bartels) over
// the C ABI in bartels_gpu.h.
//
// Matrix arguments are any column-major dense type exposing data(), rows(),
// cols() (and resize(r, c) for outputs): Eigen::MatrixXd / MatrixXi /
// VectorXd work as-is, as do the small sim::Dense<T> types below. Sparse
// outputs are sim::SparseMatrix (compressed columns, Eigen's default layout)
// and can be wrapped with Eigen::Map<Eigen::SparseMatrix<double>>.
//
// Mesh plans are cached by content (E, and V for tets, compared exactly; the
// four most recently used are kept), so repeated calls on one mesh reuse its
// pattern and a buffer reused for another mesh never meets a stale plan;
// element data is uploaded per call as in the reference. Errors throw sim::Error (the reference asserts or
// exits).
#pragma once

#include <algorithm>
#include <cstdint>
#include <list>
#include <stdexcept>
#include <string>
#include <tuple>
#include <type_traits>
#include <vector>

#include "bartels_gpu.h"

namespace sim {

struct Error : std::runtime_error {
  int status;
  Error(int s, const std::string &where)
      : std::runtime_error(where + ": " + bartels_status_string(s) + " (" + bartels_last_error() + ")"), status(s) {}
};

inline void check(int s, const char *where) {
  if (s != BARTELS_OK) throw Error(s, where);
}

enum SolverExitStatus { CONVERGED = BARTELS_CONVERGED, MAX_ITERATIONS_REACHED = BARTELS_MAX_ITERATIONS_REACHED };

// Minimal column-major dense matrix for callers without Eigen.
template <class T>
struct Dense {
  std::vector<T> v;
  int r = 0, c = 0;
  Dense() = default;
  Dense(int rows, int cols) : v((size_t)rows * cols), r(rows), c(cols) {}
  T *data() { return v.data(); }
  const T *data() const { return v.data(); }
  int rows() const { return r; }
  int cols() const { return c; }
  void resize(int rows, int cols) {
    r = rows;
    c = cols;
    v.assign((size_t)rows * cols, T(0));
  }
  T &operator()(int i, int j) { return v[i + (size_t)r * j]; }
  const T &operator()(int i, int j) const { return v[i + (size_t)r * j]; }
  T &operator()(int i) { return v[i]; }
  const T &operator()(int i) const { return v[i]; }
};
using MatrixXd = Dense<double>;
using MatrixXi = Dense<int>;
using VectorXd = Dense<double>;

// Compressed-column storage, Eigen::SparseMatrix's default layout:
// outer_ptr (n_cols + 1) indexes columns, inner_idx holds row indices. The
// Hessians and mass matrices have a symmetric pattern, so the same arrays also
// read as compressed rows; the constraint matrix P is rectangular.
struct SparseMatrix {
  int n_rows = 0, n_cols = 0;
  std::vector<int> outer_ptr, inner_idx;
  std::vector<double> values;
  int rows() const { return n_rows; }
  int cols() const { return n_cols; }
  int64_t nonZeros() const { return (int64_t)values.size(); }
};

// One context for the process (the C ABI allows one per host thread).
inline bartels_ctx context() {
  static bartels_ctx ctx = [] {
    bartels_ctx c = nullptr;
    check(bartels_ctx_create(0, &c), "bartels_ctx_create");
    return c;
  }();
  return ctx;
}

namespace detail {
// Most-recently-used list of plans keyed by (tag, nV, V values, E values).
template <class Plan>
struct PlanCache {
  struct Item {
    int tag, nV;
    std::vector<double> V;
    std::vector<int> E;
    Plan plan;
  };
  std::list<Item> items;
  template <class Make, class Destroy>
  Plan get(int tag, int nV, const double *V, size_t nVvals, const int *E, size_t nE, Make make, Destroy destroy) {
    for (auto it = items.begin(); it != items.end(); ++it) {
      if (it->tag != tag || it->nV != nV || it->V.size() != nVvals || it->E.size() != nE) continue;
      if (!std::equal(E, E + nE, it->E.begin()) || !std::equal(V, V + nVvals, it->V.begin())) continue;
      items.splice(items.begin(), items, it);
      return items.front().plan;
    }
    Plan p = make();
    items.push_front(Item{tag, nV, std::vector<double>(V, V + nVvals), std::vector<int>(E, E + nE), p});
    while (items.size() > 4) {
      destroy(items.back().plan);
      items.pop_back();
    }
    return p;
  }
};

template <class MV, class ME>
bartels_mesh_plan plan_for(const MV &V, const ME &E) {
  static PlanCache<bartels_mesh_plan> cache;
  const int nV = (int)V.rows(), nT = (int)E.rows();
  return cache.get(0, nV, V.data(), 3 * (size_t)nV, E.data(), 4 * (size_t)nT,
                   [&] {
                     bartels_mesh_plan p = nullptr;
                     check(bartels_plan_create(context(), nV, V.data(), nT, E.data(), &p), "bartels_plan_create");
                     return p;
                   },
                   [](bartels_mesh_plan p) { bartels_plan_destroy(p); });
}
template <class Out>
void copy_pattern(SparseMatrix &S, bartels_mesh_plan p, int n, int64_t nnz) {
  S.n_rows = S.n_cols = n;
  S.outer_ptr.resize(n + 1);
  S.inner_idx.resize(nnz);
  check(bartels_plan_csr_pattern(p, S.outer_ptr.data(), S.inner_idx.data()), "bartels_plan_csr_pattern");
}
// The library returns values in row order (entry (i, j) of row i). For a
// structurally symmetric pattern the same index arrays describe the columns;
// this moves each value to its mirror position so that the stored entry at
// (row inner_idx[k], column c) is H(inner_idx[k], c), as in the reference's
// column-major Eigen matrix (the two differ by FP32 rounding only).
inline void row_values_to_columns(SparseMatrix &S) {
  std::vector<double> col_vals(S.values.size());
  for (int r = 0; r < S.n_rows; ++r)
    for (int k = S.outer_ptr[r]; k < S.outer_ptr[r + 1]; ++k) {
      const int c = S.inner_idx[k];
      const int *b = S.inner_idx.data() + S.outer_ptr[c], *e = S.inner_idx.data() + S.outer_ptr[c + 1];
      const int *f = std::lower_bound(b, e, r);
      if (f == e || *f != r) throw Error(BARTELS_E_INVALID_ARG, "pattern is not structurally symmetric");
      col_vals[f - S.inner_idx.data()] = S.values[k];  // H(r, c) stored in column c at row r
    }
  S.values.swap(col_vals);
}
}  // namespace detail

// element-matrix callback replacements (src/linear_tetmesh_neohookean_dq2.cpp:22)
struct default_callback_t {};
struct simple_psd_fix_t {
  double tol = 1e-6;  // include/simple_psd_fix.h:11
};
inline simple_psd_fix_t simple_psd_fix(double tol = 1e-6) { return simple_psd_fix_t{tol}; }

// linear_tetmesh_dphi_dX, include/linear_tetmesh_dphi_dX.h
template <class MR, class MV, class ME>
void linear_tetmesh_dphi_dX(MR &dX, const MV &V, const ME &E) {
  dX.resize((int)E.rows(), 12);
  check(bartels_tetmesh_dphi_dX(context(), (int)V.rows(), V.data(), (int)E.rows(), E.data(), dX.data()),
        "bartels_tetmesh_dphi_dX");
}

#define BARTELS_SIM_MODEL(name, id)                                                                                \
  template <class MV, class ME, class MQ, class MD, class MVol, class MP>                                          \
  double linear_tetmesh_##name##_q(const MV &V, const ME &E, const MQ &q, const MD &dphidX, const MVol &volume,   \
                                   const MP &params) {                                                             \
    double e = 0;                                                                                                  \
    check(bartels_tetmesh_q(context(), detail::plan_for(V, E), id, q.data(), dphidX.data(), volume.data(),         \
                            params.data(), &e),                                                                    \
          "linear_tetmesh_" #name "_q");                                                                           \
    return e;                                                                                                      \
  }                                                                                                                \
  template <class MG, class MV, class ME, class MQ, class MD, class MVol, class MP>                                \
  void linear_tetmesh_##name##_dq(MG &g, const MV &V, const ME &E, const MQ &q, const MD &dphidX,                  \
                                  const MVol &volume, const MP &params) {                                          \
    g.resize(3 * (int)V.rows(), 1);                                                                                \
    check(bartels_tetmesh_dq(context(), detail::plan_for(V, E), id, q.data(), dphidX.data(), volume.data(),        \
                             params.data(), g.data()),                                                             \
          "linear_tetmesh_" #name "_dq");                                                                          \
  }                                                                                                                \
  template <class MV, class ME, class MQ, class MD, class MVol, class MP, class CB = default_callback_t>            \
  void linear_tetmesh_##name##_dq2(SparseMatrix &H, const MV &V, const ME &E, const MQ &q, const MD &dphidX,       \
                                   const MVol &volume, const MP &params, const CB &cb = CB()) {                    \
    bartels_mesh_plan p = detail::plan_for(V, E);                                                                  \
    int n = 0;                                                                                                     \
    int64_t nnz = 0;                                                                                               \
    check(bartels_plan_csr_size(p, &n, &nnz), "bartels_plan_csr_size");                                            \
    detail::copy_pattern<SparseMatrix>(H, p, n, nnz);                                                              \
    H.values.resize(nnz);                                                                                          \
    int psd = BARTELS_PSD_NONE;                                                                                    \
    double tol = 0.0;                                                                                              \
    if constexpr (std::is_same<CB, simple_psd_fix_t>::value) {                                                     \
      psd = BARTELS_PSD_SIMPLE_FIX;                                                                                \
      tol = cb.tol;                                                                                                \
    }                                                                                                              \
    check(bartels_tetmesh_dq2(context(), p, id, q.data(), dphidX.data(), volume.data(), params.data(), psd, tol, 0, \
                              H.values.data()),                                                                    \
          "linear_tetmesh_" #name "_dq2");                                                                         \
    detail::row_values_to_columns(H);                                                                              \
  }

BARTELS_SIM_MODEL(neohookean, BARTELS_NEOHOOKEAN)
BARTELS_SIM_MODEL(stvk, BARTELS_STVK)
BARTELS_SIM_MODEL(corotational, BARTELS_COROTATIONAL)
BARTELS_SIM_MODEL(arap, BARTELS_ARAP)
BARTELS_SIM_MODEL(linear_elasticity, BARTELS_LINEAR_ELASTICITY)
#undef BARTELS_SIM_MODEL

// ------------------------------------------------------------ pointwise laws --
// psi_<law>_F, dpsi_<law>_dF, d2psi_<law>_dF2 (include/psi_neohookean_F.h,
// include/dpsi_neohookean_dF.h, include/d2psi_neohookean_dF2.h and the StVK
// siblings): F a 3x3 column-major dense type, params 2 contiguous values; dw
// becomes 9 x 1 (dpsi/dF in the column-major flatten of F), ddw 9 x 9. Each
// call is one device round trip; bartels_pointwise_laws takes a batch.
namespace detail {
template <class MF, class MP>
void pointwise(int model, const MF &F, const MP &params, double *psi, double *dpsi, double *d2psi) {
  if (F.rows() != 3 || F.cols() != 3 || (int)(params.rows() * params.cols()) < 2)
    throw Error(BARTELS_E_INVALID_ARG, "pointwise law: F must be 3 x 3 and params hold 2 values");
  check(bartels_pointwise_laws(context(), model, 1, F.data(), params.data(), psi, dpsi, d2psi),
        "bartels_pointwise_laws");
}
}  // namespace detail

#define BARTELS_SIM_LAW(name, id)                                                  \
  template <class MF, class MP>                                                   \
  double psi_##name##_F(const MF &F, const MP &params) {                          \
    double e = 0.0;                                                               \
    detail::pointwise(id, F, params, &e, nullptr, nullptr);                       \
    return e;                                                                     \
  }                                                                               \
  template <class MG, class MF, class MP>                                         \
  void dpsi_##name##_dF(MG &dw, const MF &F, const MP &params) {                  \
    dw.resize(9, 1);                                                              \
    detail::pointwise(id, F, params, nullptr, dw.data(), nullptr);                \
  }                                                                               \
  template <class MH, class MF, class MP>                                         \
  void d2psi_##name##_dF2(MH &ddw, const MF &F, const MP &params) {               \
    ddw.resize(9, 9);                                                             \
    detail::pointwise(id, F, params, nullptr, nullptr, ddw.data());               \
  }
BARTELS_SIM_LAW(neohookean, BARTELS_NEOHOOKEAN)
BARTELS_SIM_LAW(stvk, BARTELS_STVK)
#undef BARTELS_SIM_LAW

// ----------------------------------------------------------- triangle meshes --
namespace detail {
template <class MV, class ME>
bartels_tri_plan tri_plan_for(const MV &V, const ME &E, int dim) {
  static PlanCache<bartels_tri_plan> cache;
  const int nV = (int)V.rows(), nT = (int)E.rows();
  return cache.get(dim, nV, nullptr, 0, E.data(), 3 * (size_t)nT,
                   [&] {
                     bartels_tri_plan p = nullptr;
                     check(bartels_tri_plan_create(context(), nV, nT, E.data(), dim, &p), "bartels_tri_plan_create");
                     return p;
                   },
                   [](bartels_tri_plan p) { bartels_tri_plan_destroy(p); });
}
inline void tri_pattern(SparseMatrix &S, bartels_tri_plan p) {
  int n = 0;
  int64_t nnz = 0;
  check(bartels_tri_plan_csr_size(p, &n, &nnz), "bartels_tri_plan_csr_size");
  S.n_rows = S.n_cols = n;
  S.outer_ptr.resize(n + 1);
  S.inner_idx.resize(nnz);
  S.values.resize(nnz);
  check(bartels_tri_plan_csr_pattern(p, S.outer_ptr.data(), S.inner_idx.data()), "bartels_tri_plan_csr_pattern");
}
template <class CB>
void psd_of(const CB &cb, int &psd, double &tol) {
  psd = BARTELS_PSD_NONE;
  tol = 0.0;
  if constexpr (std::is_same<CB, simple_psd_fix_t>::value) {
    psd = BARTELS_PSD_SIMPLE_FIX;
    tol = cb.tol;
  }
}
}  // namespace detail

// linear_tri2dmesh_dphi_dX, include/linear_tri2dmesh_dphi_dX.h (dX: nT x 6)
template <class MR, class MV, class ME>
void linear_tri2dmesh_dphi_dX(MR &dX, const MV &V, const ME &E) {
  dX.resize((int)E.rows(), 6);
  check(bartels_tri2dmesh_dphi_dX(context(), (int)V.rows(), V.data(), (int)E.rows(), E.data(), dX.data(), nullptr),
        "bartels_tri2dmesh_dphi_dX");
}

#define BARTELS_SIM_TRI_MODEL(name, id)                                                                            \
  template <class MV, class ME, class MQ, class MD, class MA, class MP>                                            \
  double linear_tri2dmesh_##name##_q(const MV &V, const ME &E, const MQ &q, const MD &dphidX, const MA &area,     \
                                     const MP &params) {                                                           \
    double e = 0;                                                                                                  \
    check(bartels_tri2dmesh_q(context(), detail::tri_plan_for(V, E, 2), id, q.data(), dphidX.data(), area.data(),  \
                              params.data(), &e),                                                                  \
          "linear_tri2dmesh_" #name "_q");                                                                         \
    return e;                                                                                                      \
  }                                                                                                                \
  template <class MG, class MV, class ME, class MQ, class MD, class MA, class MP>                                  \
  void linear_tri2dmesh_##name##_dq(MG &g, const MV &V, const ME &E, const MQ &q, const MD &dphidX,                \
                                    const MA &area, const MP &params) {                                            \
    g.resize(2 * (int)V.rows(), 1);                                                                                \
    check(bartels_tri2dmesh_dq(context(), detail::tri_plan_for(V, E, 2), id, q.data(), dphidX.data(), area.data(), \
                               params.data(), g.data()),                                                           \
          "linear_tri2dmesh_" #name "_dq");                                                                        \
  }                                                                                                                \
  template <class MV, class ME, class MQ, class MD, class MA, class MP, class CB = default_callback_t>              \
  void linear_tri2dmesh_##name##_dq2(SparseMatrix &H, const MV &V, const ME &E, const MQ &q, const MD &dphidX,     \
                                     const MA &area, const MP &params, const CB &cb = CB()) {                      \
    bartels_tri_plan p = detail::tri_plan_for(V, E, 2);                                                            \
    detail::tri_pattern(H, p);                                                                                     \
    int psd;                                                                                                       \
    double tol;                                                                                                    \
    detail::psd_of(cb, psd, tol);                                                                                  \
    check(bartels_tri2dmesh_dq2(context(), p, id, q.data(), dphidX.data(), area.data(), params.data(), psd, tol,   \
                                H.values.data()),                                                                  \
          "linear_tri2dmesh_" #name "_dq2");                                                                       \
    detail::row_values_to_columns(H);                                                                              \
  }

BARTELS_SIM_TRI_MODEL(neohookean, BARTELS_NEOHOOKEAN)
BARTELS_SIM_TRI_MODEL(stvk, BARTELS_STVK)
BARTELS_SIM_TRI_MODEL(corotational, BARTELS_COROTATIONAL)
BARTELS_SIM_TRI_MODEL(arap, BARTELS_ARAP)
#undef BARTELS_SIM_TRI_MODEL

// linear_tri2dmesh_linear_elasticity_dq2 (the reference has only the Hessian)
template <class MV, class ME, class MQ, class MD, class MA, class MP, class CB = default_callback_t>
void linear_tri2dmesh_linear_elasticity_dq2(SparseMatrix &H, const MV &V, const ME &E, const MQ &q, const MD &dphidX,
                                            const MA &area, const MP &params, const CB &cb = CB()) {
  bartels_tri_plan p = detail::tri_plan_for(V, E, 2);
  detail::tri_pattern(H, p);
  int psd;
  double tol;
  detail::psd_of(cb, psd, tol);
  check(bartels_tri2dmesh_dq2(context(), p, BARTELS_LINEAR_ELASTICITY, q.data(), dphidX.data(), area.data(),
                              params.data(), psd, tol, H.values.data()),
        "linear_tri2dmesh_linear_elasticity_dq2");
  detail::row_values_to_columns(H);
}

// linear_tri2dmesh_mass_matrix, include/linear_tri2dmesh_mass_matrix.h
template <class MV, class ME, class MD, class MA>
void linear_tri2dmesh_mass_matrix(SparseMatrix &M, const MV &V, const ME &E, const MD &density, const MA &area) {
  bartels_tri_plan p = detail::tri_plan_for(V, E, 2);
  detail::tri_pattern(M, p);
  check(bartels_tri2dmesh_mass_matrix(context(), p, density.data(), area.data(), M.values.data()),
        "linear_tri2dmesh_mass_matrix");
  detail::row_values_to_columns(M);
}

// linear_tri3dmesh_dphi_dX, include/linear_tri3dmesh_dphi_dX.h (dX: nT x 9)
template <class MR, class MV, class ME>
void linear_tri3dmesh_dphi_dX(MR &dX, const MV &V, const ME &E) {
  dX.resize((int)E.rows(), 9);
  check(bartels_tri3dmesh_dphi_dX(context(), (int)V.rows(), V.data(), (int)E.rows(), E.data(), dX.data(), nullptr),
        "bartels_tri3dmesh_dphi_dX");
}

// linear_tri3dmesh_stvk_dq2, include/linear_tri3dmesh_stvk_dq2.h:14-25
template <class MV, class ME, class MQ, class MD, class MN, class Mn, class MdN, class MA, class MP,
          class CB = default_callback_t>
void linear_tri3dmesh_stvk_dq2(SparseMatrix &H, const MV &V, const ME &E, const MQ &q, const MD &dphidX, const MN &N,
                               const Mn &n, const MdN &dndq, const MA &area, const MP &params, const CB &cb = CB()) {
  bartels_tri_plan p = detail::tri_plan_for(V, E, 3);
  detail::tri_pattern(H, p);
  int psd;
  double tol;
  detail::psd_of(cb, psd, tol);
  check(bartels_tri3dmesh_stvk_dq2(context(), p, q.data(), dphidX.data(), N.data(), n.data(), dndq.data(),
                                   area.data(), params.data(), psd, tol, H.values.data()),
        "linear_tri3dmesh_stvk_dq2");
  detail::row_values_to_columns(H);
}

// linear_tetmesh_mass_matrix, include/linear_tetmesh_mass_matrix.h
template <class MV, class ME, class MD, class MVol>
void linear_tetmesh_mass_matrix(SparseMatrix &M, const MV &V, const ME &E, const MD &density, const MVol &volume) {
  bartels_mesh_plan p = detail::plan_for(V, E);
  int n = 0;
  int64_t nnz = 0;
  check(bartels_plan_csr_size(p, &n, &nnz), "bartels_plan_csr_size");
  detail::copy_pattern<SparseMatrix>(M, p, n, nnz);
  M.values.resize(nnz);
  check(bartels_tetmesh_mass_matrix(context(), p, density.data(), volume.data(), M.values.data()),
        "linear_tetmesh_mass_matrix");
  detail::row_values_to_columns(M);
}

// linear_tetmesh_const_ext_force, include/linear_tetmesh_const_ext_force.h
template <class MF, class MV, class ME, class MVol, class MT>
void linear_tetmesh_const_ext_force(MF &f, const MV &V, const ME &E, const MVol &volume, const MT &traction) {
  f.resize(3 * (int)V.rows(), 1);
  check(bartels_tetmesh_const_ext_force(context(), detail::plan_for(V, E), volume.data(), traction.data(), f.data()),
        "linear_tetmesh_const_ext_force");
}

// fixed_point_constraint_matrix, include/fixed_point_constraint_matrix.h:
// P (d (nV - k) x d nV, one 1 per row at a free DOF) in compressed columns:
// column c holds row r when DOF c is the r-th free one.
template <class MV, class MI>
void fixed_point_constraint_matrix(SparseMatrix &P, const MV &V, const MI &fixed_indices) {
  int rows = 0;
  const int nfix = (int)(fixed_indices.rows() * fixed_indices.cols());
  check(bartels_fixed_point_constraint_matrix((int)V.rows(), (int)V.cols(), fixed_indices.data(), nfix, &rows,
                                              nullptr, nullptr, nullptr),
        "fixed_point_constraint_matrix");
  std::vector<int> rp(rows + 1), col(rows);
  check(bartels_fixed_point_constraint_matrix((int)V.rows(), (int)V.cols(), fixed_indices.data(), nfix, &rows,
                                              rp.data(), col.data(), nullptr),
        "fixed_point_constraint_matrix");
  P.n_rows = rows;
  P.n_cols = (int)(V.rows() * V.cols());
  P.outer_ptr.assign(P.n_cols + 1, 0);
  P.inner_idx.resize(rows);
  P.values.assign(rows, 1.0);
  for (int r = 0; r < rows; ++r) P.outer_ptr[col[r] + 1] = 1;
  for (int c = 0; c < P.n_cols; ++c) P.outer_ptr[c + 1] += P.outer_ptr[c];
  for (int r = 0; r < rows; ++r) P.inner_idx[P.outer_ptr[col[r]]] = r;
}

// find_min_vertices, include/find_min_vertices.h: appends (as the reference's
// push_back) the vertices whose coordinate dim is within tol of its minimum.
template <class MV>
void find_min_vertices(std::vector<int> &indices, const MV &V, unsigned int dim, double tol = 1e-3) {
  std::vector<int> found(V.rows() > 0 ? V.rows() : 1);
  int count = 0;
  check(bartels_find_min_vertices((int)V.rows(), V.data(), (int)dim, tol, found.data(), &count),
        "find_min_vertices");
  indices.insert(indices.end(), found.begin(), found.begin() + count);
}

// search_direction_newton_sparse, include/search_direction_newton_sparse.h:8-12.
// The solver argument selects PCG parameters (the reference's SparseLU is
// replaced by GPU PCG); returns false where solver.info() != Success.
struct PCGSolver {
  bartels_pcg_params params;
  bartels_pcg_report report{};
  PCGSolver() { bartels_pcg_default_params(&params); }
};
namespace detail {
// Compressed columns -> compressed rows (the C ABI's layout) of a square matrix.
inline void columns_to_rows(const SparseMatrix &H, std::vector<int> &rp, std::vector<int> &ci,
                            std::vector<double> &v) {
  const int n = H.n_rows;
  rp.assign(n + 1, 0);
  ci.resize(H.inner_idx.size());
  v.resize(H.values.size());
  for (int i : H.inner_idx) rp[i + 1]++;
  for (int r = 0; r < n; ++r) rp[r + 1] += rp[r];
  std::vector<int> fill(rp.begin(), rp.end() - 1);
  for (int c = 0; c < H.n_cols; ++c)  // columns in order: rows receive ascending column indices
    for (int k = H.outer_ptr[c]; k < H.outer_ptr[c + 1]; ++k) {
      const int r = H.inner_idx[k];
      ci[fill[r]] = c;
      v[fill[r]++] = H.values[k];
    }
}
}  // namespace detail

template <class MD, class MG>
bool search_direction_newton_sparse(MD &d, const MG &g, const SparseMatrix &H, PCGSolver &solver) {
  d.resize((int)g.rows(), 1);
  if (H.n_rows != H.n_cols || (int)H.outer_ptr.size() != H.n_cols + 1)
    throw Error(BARTELS_E_INVALID_ARG, "search_direction_newton_sparse: H must be square, compressed columns");
  std::vector<int> rp, ci;
  std::vector<double> v;
  detail::columns_to_rows(H, rp, ci, v);
  const int s = bartels_search_direction_newton_sparse(context(), H.rows(), rp.data(), ci.data(), v.data(),
                                                       g.data(), d.data(), &solver.params, &solver.report);
  if (s == BARTELS_E_NOT_CONVERGED) return false;
  check(s, "search_direction_newton_sparse");
  return true;
}

// linesearch_backtracking_bisection, include/linesearch_backtracking_bisection.h:23-33
template <class MX, class Objective>
SolverExitStatus linesearch_backtracking_bisection(MX &x, const MX &d, const Objective &f, const MX &g,
                                                   unsigned int max_iterations, double alpha, double c, double p) {
  struct Thunk {
    const Objective *f;
    int rows, cols;
    static double call(const double *xp, int n, void *u) {
      auto *t = static_cast<Thunk *>(u);
      MX tmp;
      tmp.resize(t->rows, t->cols);
      for (int i = 0; i < n; ++i) tmp.data()[i] = xp[i];
      return (*t->f)(tmp);
    }
  } th{&f, (int)x.rows(), (int)x.cols()};
  int status = 0;
  check(bartels_linesearch_backtracking_bisection((int)(x.rows() * x.cols()), x.data(), d.data(), &Thunk::call, &th,
                                                  g.data(), (int)max_iterations, alpha, c, p, &status, nullptr),
        "linesearch_backtracking_bisection");
  return status == BARTELS_CONVERGED ? CONVERGED : MAX_ITERATIONS_REACHED;
}

}  // namespace sim
