// oracle/quadprog_ref.cpp -- C entry point over the reference's vendored
// QuadProg++ (src/MPRGPSolver/SimpleQP/QuadProg.cpp, Array.cpp).
//
// TEST INFRASTRUCTURE ONLY.  oracle/build_ref.sh compiles this file together
// with those two reference sources, where they lie in the read-only reference
// tree, into oracle/_ref/libquadprog_ref.so.  Nothing is copied into this
// repository.  The CPU tests use it to pin the oracle: the reference's
// GeneralConProjector solves its projection and BETA sub-problems with
// exactly this routine (MPRGPProjection.h:427, :465), through the wrapper
// solveQP (SimpleQP.h:17-48), whose problem statement this function keeps:
//
//     min 0.5 x^T A x - b^T x   s.t.   J x >= c0
//
// mapped to QuadProg++'s  min 0.5 x^T G x + g0^T x,  CI^T x + ci0 >= 0  with
// G = A, g0 = -b, CI = J^T, ci0 = -c0 (SimpleQP.h:32-41).
#include <limits>

#include "QuadProg.h"

extern "C" double ref_solve_qp(int n, const double *A, const double *b, int m,
                               const double *J, const double *c0, double *x) {
  QuadProgPP::Matrix<double> G(n, n);
  QuadProgPP::Vector<double> g0(n);
  QuadProgPP::Matrix<double> CE(n, 0);
  QuadProgPP::Vector<double> ce0(0);
  QuadProgPP::Matrix<double> CI(n, m);
  QuadProgPP::Vector<double> ci0(m);
  for (int r = 0; r < n; ++r) {
    g0[r] = -b[r];
    for (int c = 0; c < n; ++c) G[r][c] = A[r * n + c];
    for (int c = 0; c < m; ++c) CI[r][c] = J[c * n + r];
  }
  for (int c = 0; c < m; ++c) ci0[c] = -c0[c];
  QuadProgPP::Vector<double> x0(n);
  const double f = QuadProgPP::QuadProg::solve_quadprog(G, g0, CE, ce0, CI, ci0, x0);
  for (int r = 0; r < n; ++r) x[r] = x0[r];
  return f;
}
