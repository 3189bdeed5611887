// include/mprgp/MPRGPSolver.h -- drop-in C++ façade of the reference's
// src/MPRGPSolver/MPRGPSolver.h over the GB300 C ABI (include/mprgp_gpu.h).
//
// Same namespace, class names and solve() signatures as the reference:
//   MPRGPLowerBound<T>::solve(A, B, L, x, tol, max_it)           (:503-517)
//   MPRGPBoxBound<T>::solve(A, B, L, U, x, tol, max_it)          (:520-535)
//   MPRGPDecoupledCon<T>::solve<MAT, preconditioned>(A, B, projector, x, tol,
//       max_it, name, ev) / solve(A, B, J, c, x, ...) / solve(file, x, ...)
//                                                                (:538-590)
//   MPRGPGeneralCon<T>::solve<MAT, preconditioned>(...)           (:593-626)
//   MPRGP<T,MAT,PROJ,PRECOND> / MPRGPMonotonic<...> with solve(x),
//       iterationsOut(), residualOut(), printSolveInfo()          (:345-456)
//   FixedSparseMatrix<T> (multiply, funcValue, rows, diag)        (:459-500)
// Return codes as the reference: 0 converged, -1 not converged; other
// negative values are the C ABI's errors (no CUDA device, invalid shape...).
//
// Every solve runs on the GPU: A (n x n, n = 3 * vertices; other n are padded
// with one decoupled unknown) is converted to 3x3 blocks, the rows of J to
// per-vertex planes (each row must touch one vertex's three columns, at most
// three rows per vertex), and x, the face and ev come back into the caller's
// objects.  Link with libmprgp_gb300.so.
#pragma once

#include <cstdio>
#include <iostream>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "../mprgp_gpu.h"
#include "MPRGPProjection.h"
#include "MPRGPUtility.h"

namespace MATH {

// FixedSparseMatrix (MPRGPSolver.h:459-500): holds A; its host methods keep
// the reference's MAT concept for callers that use them directly.
template <typename T>
class FixedSparseMatrix {
 public:
  explicit FixedSparseMatrix(const SparseMatrix<T> &M) : A(M), diag_A(M.rows()) {
    for (int i = 0; i < M.rows(); ++i) diag_A[i] = M.coeff(i, i);
  }
  void multiply(const Vec<T> &x, Vec<T> &y) const { A.multiply(x, y); }
  T funcValue(const Vec<T> &x, const Vec<T> &b) const {
    Vec<T> ax;
    A.multiply(x, ax);
    T s = 0, t = 0;
    for (size_t i = 0; i < x.size(); ++i) {
      s += x[i] * ax[i];
      t += x[i] * b[i];
    }
    return (T)0.5 * s - t;
  }
  int rows() const { return A.rows(); }
  double diag(int i) const { return diag_A[i]; }
  const SparseMatrix<T> &getMatrix() const { return A; }

 private:
  SparseMatrix<T> A;
  Vec<T> diag_A;
};

namespace gpu {

// Statistics of the last solve on this thread (the reference prints them
// through printSolveInfo, MPRGPSolver.h:138-145).
inline mprgp_stats &last_stats() {
  static thread_local mprgp_stats s{};
  return s;
}

// One context per (host thread, device) for the façade.
inline int &device() {
  static thread_local int d = 0;
  return d;
}
inline mprgp_context *context() {
  static thread_local std::map<int, mprgp_context *> ctx;
  auto it = ctx.find(device());
  if (it != ctx.end()) return it->second;
  mprgp_context *c = nullptr;
  const int rc = mprgp_context_create(device(), &c);
  if (rc != MPRGP_OK) return nullptr;
  ctx[device()] = c;
  return c;
}

template <typename T>
const SparseMatrix<T> &matrix_of(const FixedSparseMatrix<T> &A) {
  return A.getMatrix();
}
template <typename T>
const SparseMatrix<T> &matrix_of(const SparseMatrix<T> &A) {
  return A;
}

// The 3x3-block form of an n x n scalar CSR over nv = ceil(n / 3) vertices,
// with the map from each scalar entry to its block value.  Padded unknowns
// get a unit-free diagonal equal to the smallest positive diagonal entry of
// A (never above the spectral radius) and no coupling.  The FEM driver
// re-solves with the same sparsity every Newton iteration
// (MprgpFemSolver.cpp:521-533), so the pattern is kept per thread and a
// matrix with the same pattern only refills the values.
struct BlockPattern {
  std::vector<int> sptr, sidx;  // the scalar pattern the blocks were built for
  int n = -1, nv = 0;
  std::vector<int> row_ptr, cols;
  std::vector<size_t> where;  // scalar entry k -> its block value
  std::vector<size_t> diag;   // scalar entries on the diagonal
  std::vector<size_t> pad;    // block values of the padded unknowns' diagonal
  std::vector<double> vals;
  long long builds = 0, refills = 0;
};
inline BlockPattern &block_pattern() {
  static thread_local BlockPattern p;
  return p;
}

template <typename T>
void build_pattern(const SparseMatrix<T> &A, BlockPattern &P) {
  const int n = A.rows();
  const auto &ptr = A.outerIndex();
  const auto &idx = A.innerIndex();
  P.n = n;
  P.nv = (n + 2) / 3;
  P.sptr = ptr;
  P.sidx = idx;
  P.row_ptr.assign(P.nv + 1, 0);
  P.cols.clear();
  P.where.assign(idx.size(), 0);
  P.diag.clear();
  P.pad.clear();
  std::vector<int> bc;
  for (int v = 0; v < P.nv; ++v) {
    bc.clear();
    for (int r = 3 * v; r < std::min(n, 3 * v + 3); ++r)
      for (int k = ptr[r]; k < ptr[r + 1]; ++k) bc.push_back(idx[k] / 3);
    bc.push_back(v);
    std::sort(bc.begin(), bc.end());
    bc.erase(std::unique(bc.begin(), bc.end()), bc.end());
    const size_t base = P.cols.size();
    P.cols.insert(P.cols.end(), bc.begin(), bc.end());
    auto slot = [&](int cb) {
      return base + (size_t)(std::lower_bound(bc.begin(), bc.end(), cb) - bc.begin());
    };
    for (int i = 0; i < 3; ++i) {
      const int r = 3 * v + i;
      if (r >= n) {
        P.pad.push_back(9 * slot(v) + 4 * i);
        continue;
      }
      for (int k = ptr[r]; k < ptr[r + 1]; ++k) {
        P.where[k] = 9 * slot(idx[k] / 3) + 3 * i + (idx[k] % 3);
        if (idx[k] == r) P.diag.push_back((size_t)k);
      }
    }
    P.row_ptr[v + 1] = (int)P.cols.size();
  }
  ++P.builds;
}

// The block values of A on pattern P: entries summed in scalar order.
template <typename T>
void fill_values(const SparseMatrix<T> &A, BlockPattern &P) {
  const auto &val = A.values();
  P.vals.assign(9 * P.cols.size(), 0.0);
  for (size_t k = 0; k < P.where.size(); ++k) P.vals[P.where[k]] += (double)val[k];
  double dmin = 0.0;
  bool first = true;
  for (size_t k : P.diag) {  // the smallest positive diagonal entry
    const double d = (double)val[k];
    if (d > 0 && (first || d < dmin)) {
      dmin = d;
      first = false;
    }
  }
  if (first) dmin = 1.0;
  for (size_t q : P.pad) P.vals[q] = dmin;
}

// A's blocks, rebuilding the pattern only when A's sparsity changed.
template <typename T>
const BlockPattern &to_bsr(const SparseMatrix<T> &A) {
  BlockPattern &P = block_pattern();
  if (P.n != A.rows() || P.sptr != A.outerIndex() || P.sidx != A.innerIndex())
    build_pattern(A, P);
  else
    ++P.refills;
  fill_values(A, P);
  return P;
}

// Rows of J (J x >= c) -> per-vertex planes (n, p = -c) in plane_ptr order;
// order[k] is the row of J behind plane k.  Returns false if a row touches
// more than one vertex.
template <typename T>
bool to_planes(const SparseMatrix<T> &J, const Vec<T> &c, int nv, std::vector<int> &plane_ptr,
               std::vector<double> &planes, std::vector<int> &order) {
  const auto &ptr = J.outerIndex();
  const auto &idx = J.innerIndex();
  const auto &val = J.values();
  std::vector<std::vector<int>> rows(nv);
  for (int r = 0; r < J.rows(); ++r) {
    if (ptr[r + 1] == ptr[r]) return false;
    const int v = idx[ptr[r]] / 3;
    for (int k = ptr[r]; k < ptr[r + 1]; ++k)
      if (idx[k] / 3 != v) return false;
    rows[v].push_back(r);
  }
  plane_ptr.assign(nv + 1, 0);
  planes.clear();
  order.clear();
  for (int v = 0; v < nv; ++v) {
    for (int r : rows[v]) {
      double n3[3] = {0, 0, 0};
      for (int k = ptr[r]; k < ptr[r + 1]; ++k) n3[idx[k] % 3] += (double)val[k];
      planes.insert(planes.end(), {n3[0], n3[1], n3[2], -(double)c[r]});
      order.push_back(r);
    }
    plane_ptr[v + 1] = (int)order.size();
  }
  return true;
}

// The façade's one solve: kind / precond per mprgp_gpu.h, x in and out.
template <typename T>
int solve(const SparseMatrix<T> &A, const Vec<T> &B, const SparseMatrix<T> *J, const Vec<T> *c,
          const Vec<T> *L, const Vec<T> *U, Vec<T> &x, int kind, int algorithm, int precond,
          T tol, int max_it, int project_x0, Vec<T> *ev, std::vector<char> *face) {
  mprgp_context *ctx = context();
  if (!ctx) return MPRGP_NO_DEVICE;
  const int n = A.rows();
  if (A.cols() != n || (int)B.size() != n || (int)x.size() != n) return MPRGP_INVALID;
  const BlockPattern &P = to_bsr(A);
  const int nv = P.nv;
  const int np = 3 * nv;
  std::vector<double> b(np, 0.0), xx(np, 0.0), l, u, evv;
  for (int i = 0; i < n; ++i) {
    b[i] = (double)B[i];
    xx[i] = (double)x[i];
  }
  std::vector<int> plane_ptr, order;
  std::vector<double> planes;
  if (kind >= MPRGP_KIND_DECOUPLED) {
    if (!to_planes(*J, *c, nv, plane_ptr, planes, order)) return MPRGP_INVALID;
  } else {
    l.assign(np, -1e300);
    u.assign(np, 1e300);
    for (int i = 0; i < n; ++i) {
      l[i] = (double)(*L)[i];
      if (U) u[i] = (double)(*U)[i];
    }
  }
  mprgp_options opt;
  mprgp_default_options(&opt);
  opt.tol = (double)tol;
  opt.max_it = max_it;
  opt.kind = kind;
  opt.algorithm = algorithm;
  opt.precond = precond;
  opt.project_x0 = project_x0;
  if (ev && (int)ev->size() == n) {  // specRad warm start (MPRGPSolver.h:47-48)
    evv.assign(np, 0.0);
    for (int i = 0; i < n; ++i) evv[i] = (double)(*ev)[i];
    opt.use_ev = 1;
  } else if (ev) {
    evv.assign(np, 0.0);
  }
  const size_t m = kind >= MPRGP_KIND_DECOUPLED ? order.size() : (size_t)np;
  std::vector<unsigned char> f(std::max<size_t>(m, 1), 0);
  mprgp_stats st{};
  const int rc = mprgp_solve_bsr(ctx, nv, (int)P.cols.size(), P.row_ptr.data(), P.cols.data(),
                                 P.vals.data(), b.data(), plane_ptr.empty() ? nullptr : plane_ptr.data(),
                                 planes.empty() ? nullptr : planes.data(),
                                 l.empty() ? nullptr : l.data(), u.empty() ? nullptr : u.data(), &opt,
                                 xx.data(), f.data(), ev ? evv.data() : nullptr, &st);
  last_stats() = st;
  if (rc < MPRGP_NOT_CONVERGED) return rc;
  for (int i = 0; i < n; ++i) x[i] = (T)xx[i];
  if (ev && st.ev_updated) {
    ev->resize(n);
    for (int i = 0; i < n; ++i) (*ev)[i] = (T)evv[i];
  }
  if (face) {
    if (kind >= MPRGP_KIND_DECOUPLED) {
      face->assign(order.size(), 0);
      for (size_t k = 0; k < order.size(); ++k) (*face)[order[k]] = (char)f[k];
    } else {
      face->assign(n, 0);
      for (int i = 0; i < n; ++i) (*face)[i] = (char)f[i];
    }
  }
  return rc;
}

template <typename PROJ>
struct kind_of;

}  // namespace gpu

// MPRGP solver for lower bound constraints x >= L (MPRGPSolver.h:503-517).
template <typename T = double>
class MPRGPLowerBound {
 public:
  template <typename MAT>
  static int solve(const MAT &A, const Vec<T> &B, const Vec<T> &L, Vec<T> &x,
                   const T tol = 1e-3, const int max_it = 1000) {
    return gpu::solve<T>(gpu::matrix_of(A), B, nullptr, nullptr, &L, nullptr, x,
                         MPRGP_KIND_LOWER, MPRGP_ALG_DEFAULT, MPRGP_PRECOND_DEFAULT, tol, max_it,
                         0, nullptr, nullptr);
  }
};

// MPRGP solver for box constraints H >= x >= L (MPRGPSolver.h:520-535).
template <typename T = double>
class MPRGPBoxBound {
 public:
  template <typename MAT>
  static int solve(const MAT &A, const Vec<T> &B, const Vec<T> &L, const Vec<T> &U, Vec<T> &x,
                   const T tol = 1e-3, const int max_it = 1000) {
    return gpu::solve<T>(gpu::matrix_of(A), B, nullptr, nullptr, &L, &U, x, MPRGP_KIND_BOX,
                         MPRGP_ALG_DEFAULT, MPRGP_PRECOND_DEFAULT, tol, max_it, 0, nullptr,
                         nullptr);
  }
};

// Decoupled collision constraints J x >= c, J J^T diagonal (MPRGPSolver.h:538-590).
template <typename T = double>
class MPRGPDecoupledCon {
 public:
  template <typename MAT, bool preconditioned = true>
  static int solve(const MAT &A, const Vec<T> &B, DecoupledConProjector<T> &projector, Vec<T> &x,
                   const T tol = 1e-3, const int max_it = 1000,
                   const std::string solver_name = "MPRGP", Vec<T> *ev = nullptr) {
    (void)solver_name;
    return gpu::solve<T>(gpu::matrix_of(A), B, &projector.getConMatrix(), &projector.rhs(),
                         nullptr, nullptr, x, MPRGP_KIND_DECOUPLED, MPRGP_ALG_DEFAULT,
                         preconditioned ? MPRGP_PRECOND_DEFAULT : MPRGP_PRECOND_NONE, tol, max_it,
                         0, ev, &projector.faceRef());
  }
  template <typename MAT, bool preconditioned = true>
  static int solve(const MAT &A, const Vec<T> &B, const SparseMatrix<T> &J, const Vec<T> &c,
                   Vec<T> &x, const T tol = 1e-3, const int max_it = 1000,
                   const std::string solver_name = "MPRGP", Vec<T> *ev = nullptr) {
    (void)solver_name;
    return gpu::solve<T>(gpu::matrix_of(A), B, &J, &c, nullptr, nullptr, x,
                         MPRGP_KIND_DECOUPLED, MPRGP_ALG_DEFAULT,
                         preconditioned ? MPRGP_PRECOND_DEFAULT : MPRGP_PRECOND_NONE, tol, max_it,
                         1, ev, nullptr);
  }
  template <bool preconditioned = true>
  static int solve(const std::string file_name, Vec<T> &x, const T tol = 1e-3,
                   const int max_it = 1000, const std::string solver_name = "MPRGP",
                   Vec<T> *ev = nullptr) {
    SparseMatrix<T> A, J;
    Vec<T> B, c;
    if (!loadQP(A, B, J, c, x, file_name)) return -1;  // reference returns -1 too
    return solve<SparseMatrix<T>, preconditioned>(A, B, J, c, x, tol, max_it, solver_name, ev);
  }
};

// General collision constraints J x >= c (MPRGPSolver.h:593-626).
template <typename T = double>
class MPRGPGeneralCon {
 public:
  template <typename MAT, bool preconditioned = true>
  static int solve(const MAT &A, const Vec<T> &B, GeneralConProjector<T> &projector, Vec<T> &x,
                   const T tol = 1e-3, const int max_it = 1000,
                   const std::string solver_name = "MPRGP", Vec<T> *ev = nullptr) {
    (void)solver_name;
    return gpu::solve<T>(gpu::matrix_of(A), B, &projector.getConMatrix(), &projector.rhs(),
                         nullptr, nullptr, x, MPRGP_KIND_PLANES, MPRGP_ALG_DEFAULT,
                         preconditioned ? MPRGP_PRECOND_DEFAULT : MPRGP_PRECOND_NONE, tol, max_it,
                         0, ev, &projector.faceRef());
  }
  template <typename MAT, bool preconditioned = true>
  static int solve(const MAT &A, const Vec<T> &B, const SparseMatrix<T> &J, const Vec<T> &c,
                   Vec<T> &x, const T tol = 1e-3, const int max_it = 1000,
                   const std::string solver_name = "MPRGP", Vec<T> *ev = nullptr) {
    (void)solver_name;
    return gpu::solve<T>(gpu::matrix_of(A), B, &J, &c, nullptr, nullptr, x, MPRGP_KIND_PLANES,
                         MPRGP_ALG_DEFAULT,
                         preconditioned ? MPRGP_PRECOND_DEFAULT : MPRGP_PRECOND_NONE, tol, max_it,
                         1, ev, nullptr);
  }
};

namespace gpu {
template <typename T>
struct kind_of<LowerBoundProjector<T>> { static constexpr int value = MPRGP_KIND_LOWER; };
template <typename T>
struct kind_of<BoxBoundProjector<T>> { static constexpr int value = MPRGP_KIND_BOX; };
template <typename T>
struct kind_of<DecoupledConProjector<T>> { static constexpr int value = MPRGP_KIND_DECOUPLED; };
template <typename T>
struct kind_of<GeneralConProjector<T>> { static constexpr int value = MPRGP_KIND_PLANES; };

template <typename T, typename PROJ>
int solve_with(const SparseMatrix<T> &A, const Vec<T> &B, PROJ &proj, Vec<T> &x, int alg,
               int precond, T tol, int max_it, Vec<T> *ev) {
  constexpr int kind = kind_of<PROJ>::value;
  if constexpr (kind >= MPRGP_KIND_DECOUPLED) {
    return solve<T>(A, B, &proj.getConMatrix(), &proj.rhs(), nullptr, nullptr, x, kind, alg,
                    precond, tol, max_it, 0, ev, &proj.faceRef());
  } else if constexpr (kind == MPRGP_KIND_BOX) {
    return solve<T>(A, B, nullptr, nullptr, &proj.lower(), &proj.upper(), x, kind, alg, precond,
                    tol, max_it, 0, ev, &proj.face());
  } else {
    return solve<T>(A, B, nullptr, nullptr, &proj.lower(), nullptr, x, kind, alg, precond, tol,
                    max_it, 0, ev, &proj.face());
  }
}
}  // namespace gpu

// The generic solver classes (MPRGPSolver.h:345-456): MPRGP runs the plain
// variant (ratio test alpha_f), MPRGPMonotonic the monotone one.
template <typename T, typename MAT, typename PROJ, typename PRECOND, int ALG>
class MPRGPGpuSolver {
 public:
  MPRGPGpuSolver(const MAT &A, const Vec<T> &B, PRECOND &precond, PROJ &projector,
                 const int max_it = 1000, const T tol = 1e-3, Vec<T> *ev = nullptr)
      : A(A), B(B), projector(projector), max_it(max_it), tol(tol), ev(ev) {
    (void)precond;
  }
  int solve(Vec<T> &result) {
    code = gpu::solve_with<T>(gpu::matrix_of(A), B, projector, result, ALG,
                              PRECOND::engine_precond, tol, max_it, ev);
    return code;
  }
  void setName(const std::string n) { name = n; }
  size_t iterationsOut() const { return (size_t)gpu::last_stats().iterations; }
  T residualOut() const { return (T)gpu::last_stats().residual; }
  void printSolveInfo() const {
    const mprgp_stats &s = gpu::last_stats();
    std::cout << name << " cg steps: " << s.num_cg << "\n"
              << name << " exp steps: " << s.num_exp << "\n"
              << name << " prop steps: " << s.num_prop << "\n"
              << name << " total iter: " << s.iterations << "\n"
              << name << " residual: " << s.residual << "\n"
              << name << " constraints: " << s.active << std::endl;
  }

 private:
  const MAT &A;
  const Vec<T> &B;
  PROJ &projector;
  int max_it;
  T tol;
  Vec<T> *ev;
  int code = -1;
  std::string name = "MPRGP";
};

template <typename T, typename MAT, typename PROJ, typename PRECOND>
using MPRGP = MPRGPGpuSolver<T, MAT, PROJ, PRECOND, MPRGP_ALG_PLAIN>;
template <typename T, typename MAT, typename PROJ, typename PRECOND>
using MPRGPMonotonic = MPRGPGpuSolver<T, MAT, PROJ, PRECOND, MPRGP_ALG_MONOTONE>;

}  // namespace MATH
