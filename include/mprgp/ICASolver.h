// include/mprgp/ICASolver.h -- drop-in C++ façade of the reference's
// src/MPRGPSolver/ICASolver.h (class ICASolver, :287-463) over the GB300 C
// ABI (mprgp_ica_solve).
//
// Same class name, constructor defaults and methods as the reference:
//   ICASolver(max_it = 1000, tol = 1e-4, gs_max_it = 20, gs_tol = 1e-3)
//   reset(A, r) / reset(A)                      (:292-350; r = 0 for reset(A))
//   bool solve(J, p, x)                         (:352-396)
//   getResidual(), getIterations(), getLambda(), setName(), printSolveInfo()
// for A x = r + J^T lambda, 0 <= lambda _|_ J x - p >= 0.  A is n x n with
// n a multiple of 3 (the reference asserts it, :311); each row of J must
// touch one vertex's three columns, at most three rows per vertex (plane
// constraints).  The solve runs on the GPU; x and lambda come back into the
// caller's vectors, lambda in J's row order.
#pragma once

#include <iostream>
#include <string>
#include <vector>

#include "MPRGPSolver.h"

namespace MATH {

class ICASolver {
 public:
  ICASolver(const int max_it = 1000, const double tol = 1e-4, const int gs_max_it = 20,
            const double gs_tol = 1e-3)
      : max_it(max_it), tol(tol), gs_max_it(gs_max_it), gs_tol(gs_tol), name("ICASolver") {}

  void reset(const SparseMatrix<double> &A, const Vec<double> &r) {
    pA = &A;
    R = r;
  }
  void reset(const SparseMatrix<double> &A) {
    pA = &A;
    R.assign(A.rows(), 0.0);
  }

  // false when the residual did not reach tol in max_it iterations, or when
  // the call could not run (no device, J not in plane form): see lastCode().
  bool solve(const SparseMatrix<double> &J, const Vec<double> &p, Vec<double> &x) {
    code = MPRGP_INVALID;
    if (!pA || pA->rows() % 3 != 0 || pA->cols() != pA->rows() || (int)R.size() != pA->rows() ||
        (int)x.size() != pA->rows() || J.cols() != pA->rows() || (int)p.size() != J.rows())
      return false;
    mprgp_context *ctx = gpu::context();
    if (!ctx) {
      code = MPRGP_NO_DEVICE;
      return false;
    }
    const gpu::BlockPattern &P = gpu::to_bsr(*pA);
    const int nv = P.nv;
    std::vector<int> plane_ptr, order;
    std::vector<double> planes;
    if (!gpu::to_planes(J, p, nv, plane_ptr, planes, order)) return false;
    std::vector<double> xx(x.begin(), x.end()), lam(std::max<size_t>(order.size(), 1), 0.0);
    mprgp_ica_stats st{};
    code = mprgp_ica_solve(ctx, nv, (int)P.cols.size(), P.row_ptr.data(), P.cols.data(), P.vals.data(),
                           R.data(), plane_ptr.data(), planes.empty() ? nullptr : planes.data(),
                           xx.data(), lam.data(), max_it, tol, gs_max_it, gs_tol, &st);
    if (code < MPRGP_NOT_CONVERGED) return false;
    x.assign(xx.begin(), xx.end());
    lambda.assign(J.rows(), 0.0);
    for (size_t k = 0; k < order.size(); ++k) lambda[order[k]] = lam[k];
    iterations = st.iterations;
    residual = st.residual;
    return st.converged != 0;
  }

  double getResidual() const { return residual; }
  int getIterations() const { return iterations; }
  const Vec<double> &getLambda() const { return lambda; }
  int lastCode() const { return code; }
  void setName(const std::string n) { name = n; }
  void printSolveInfo(const SparseMatrix<double> &, const SparseMatrix<double> &,
                      const Vec<double> &, const Vec<double> &) const {
    std::cout << name << " residual: " << residual << "\n"
              << name << " iterations: " << iterations << "\n";
  }

 protected:
  const int max_it;
  const double tol;
  const int gs_max_it;
  const double gs_tol;
  std::string name;
  const SparseMatrix<double> *pA = nullptr;
  Vec<double> R, lambda;
  int iterations = -1, code = MPRGP_OK;
  double residual = -1.0;
};

}  // namespace MATH
