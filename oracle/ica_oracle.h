// oracle/ica_oracle.h -- CPU restatement of the reference ICA contact solver.
//
// TEST INFRASTRUCTURE ONLY (like mprgp_oracle.h): loaded by tests/ through
// liboracle.so; the product path never links it.
//
// Restates src/MPRGPSolver/ICASolver.h:
//   ICASolver::reset(A, r)  :296-350  A = La + Da + Ua by 3x3 blocks, Da^-1
//   ICASolver::solve(J,p,x) :352-393  the ICA iteration
//   GaussSeidel<true>       :20-118   projected Gauss-Seidel (PGS) on
//                                      B = J Da^-1 J^T, warm-started
// for the problem  A x = r + J^T lambda,  0 <= lambda _|_ J x - p >= 0,
// with A in 3x3-block row form (BSR, 9 values per block, row-major) and J
// given as per-vertex planes: a plane (nx, ny, nz, q) of vertex v is the row
// n at v's three columns with p = -q (the plane n.x + q >= 0).
//
// Operation order.  The reference evaluates these sums through Eigen (not
// vendored, no version pinned), whose summation order is an implementation
// detail; this restatement fixes one: every sum runs in ascending column
// (or constraint) order, a 3x3 inverse is the adjugate over the determinant
// expanded along row 0, and nothing is contracted into fused multiply-adds
// (the oracle is built with -ffp-contract=off).  The GPU solver performs the
// same operations in the same order, so its iterates are bitwise equal to
// these; against the reference itself parity is unpinned (no ICA fixture of
// the reference ships: the QP files named in test_case/MPRGP_ICA_Compare.cpp
// are absent).
//
// Structure used (exact, not an approximation):
//   * J Da^-1 J^T couples two constraints only when they sit on the same
//     vertex (Da^-1 is block diagonal), so B is block diagonal by vertex and
//     the PGS sweep over all rows equals independent sweeps per vertex, each
//     over that vertex's rows in ascending order.
//   * The 3x3-block Gauss-Seidel sweep (:378-388) reads, for block row v, the
//     new x of every block column u < v (La) and the old x of u > v (Ua);
//     its result does not depend on the order in which independent block
//     rows are processed, which is what the GPU's level schedule uses.
#pragma once

#include <cmath>
#include <vector>

namespace oracle {

struct IcaStats {
  int iterations = 0;      // ICA iterations run (the reference's `iterations`)
  int converged = 0;       // residual <= tol reached
  double residual = 0.0;   // ||A x - r - J^T lambda||
  long long pgs_sweeps = 0;  // projected Gauss-Seidel sweeps over all iterations
};

// 3x3 inverse: adjugate / det, det expanded along row 0; m row-major.
inline void inverse3(const double *m, double *inv) {
  const double a = m[0], b = m[1], c = m[2], d = m[3], e = m[4], f = m[5], g = m[6], h = m[7],
               i = m[8];
  const double c00 = e * i - f * h, c01 = f * g - d * i, c02 = d * h - e * g;
  const double det = (a * c00 + b * c01) + c * c02;
  const double s = 1.0 / det;
  inv[0] = c00 * s;
  inv[1] = (c * h - b * i) * s;
  inv[2] = (b * f - c * e) * s;
  inv[3] = c01 * s;
  inv[4] = (a * i - c * g) * s;
  inv[5] = (c * d - a * f) * s;
  inv[6] = c02 * s;
  inv[7] = (b * g - a * h) * s;
  inv[8] = (a * e - b * d) * s;
}

// y = M v for a 3x3 row-major M, each row summed left to right.
inline void mul3(const double *M, const double *v, double *y) {
  for (int k = 0; k < 3; ++k) y[k] = (M[3 * k] * v[0] + M[3 * k + 1] * v[1]) + M[3 * k + 2] * v[2];
}

// Solves with the reference's defaults gs_max_it = 20, gs_tol = 1e-3 unless
// given.  x: initial guess in, solution out (3 nv); lambda: one per plane.
inline IcaStats ica_solve(int nv, const int *row_ptr, const int *cols, const double *vals,
                          const double *r, const int *plane_ptr, const double *planes,
                          double *x, double *lambda, int max_it, double tol, int gs_max_it,
                          double gs_tol) {
  const int n = 3 * nv, m = plane_ptr[nv];
  // reset(A, r) (:296-350): Da^-1 per block row.
  std::vector<double> inv(9 * (size_t)nv, 0.0);
  for (int v = 0; v < nv; ++v)
    for (int k = row_ptr[v]; k < row_ptr[v + 1]; ++k)
      if (cols[k] == v) inverse3(vals + 9 * (size_t)k, &inv[9 * (size_t)v]);
  // B = J Da^-1 J^T within each vertex: B_ij = n_i . (Da^-1 n_j); invD = 1/B_ii.
  std::vector<double> Bv(9 * (size_t)nv, 0.0);  // per vertex, up to 3x3 (local rows)
  for (int v = 0; v < nv; ++v) {
    const int q0 = plane_ptr[v], nq = plane_ptr[v + 1] - q0;
    for (int j = 0; j < nq; ++j) {
      double t[3];
      mul3(&inv[9 * (size_t)v], planes + 4 * (size_t)(q0 + j), t);
      for (int i = 0; i < nq; ++i) {
        const double *ni = planes + 4 * (size_t)(q0 + i);
        Bv[9 * (size_t)v + 3 * i + j] = (ni[0] * t[0] + ni[1] * t[1]) + ni[2] * t[2];
      }
    }
  }
  std::vector<double> c(m), pre(m), rhs(n), w(n);
  for (int q = 0; q < m; ++q) lambda[q] = 0.0;
  IcaStats st;
  int it = 0;
  for (; it < max_it; ++it) {
    // c = p + J (Da^-1 (LaUa x - r))                                  (:371)
    for (int v = 0; v < nv; ++v) {
      double u[3];
      for (int a = 0; a < 3; ++a) {
        double acc = 0.0;
        for (int k = row_ptr[v]; k < row_ptr[v + 1]; ++k) {
          if (cols[k] == v) continue;
          const double *blk = vals + 9 * (size_t)k;
          const double *xc = x + 3 * (size_t)cols[k];
          for (int b = 0; b < 3; ++b) acc = acc + blk[3 * a + b] * xc[b];
        }
        u[a] = acc - r[3 * v + a];
      }
      double wv[3];
      mul3(&inv[9 * (size_t)v], u, wv);
      for (int q = plane_ptr[v]; q < plane_ptr[v + 1]; ++q) {
        const double *pl = planes + 4 * (size_t)q;
        c[q] = -pl[3] + ((pl[0] * wv[0] + pl[1] * wv[1]) + pl[2] * wv[2]);
      }
    }
    // PGS->solve(c, lambda) (:372; GaussSeidel::solve :67-105)
    for (int s = 0; s < gs_max_it; ++s) {
      ++st.pgs_sweeps;
      double ss = 0.0;
      for (int v = 0; v < nv; ++v) {
        const int q0 = plane_ptr[v], nq = plane_ptr[v + 1] - q0;
        const double *B = &Bv[9 * (size_t)v];
        double old[3] = {0, 0, 0};
        for (int i = 0; i < nq; ++i) old[i] = lambda[q0 + i];
        for (int i = 0; i < nq; ++i) {
          double ub = 0.0;  // (Ub lambda)_i with the sweep's starting lambda
          for (int j = i + 1; j < nq; ++j) ub = ub + B[3 * i + j] * old[j];
          double rr = c[q0 + i] - ub;
          for (int j = 0; j < i; ++j) rr -= lambda[q0 + j] * B[3 * i + j];
          double l = rr * (1.0 / B[3 * i + i]);
          lambda[q0 + i] = l > 0 ? l : 0;
        }
        for (int i = 0; i < nq; ++i) {
          const double d = lambda[q0 + i] - old[i];
          ss = ss + d * d;
        }
      }
      if (std::sqrt(ss) <= gs_tol) break;
    }
    // rhs = J^T lambda - Ua x + r (:374); then the 3x3 block sweep (:377-388)
    for (int v = 0; v < nv; ++v) {
      double jl[3] = {0, 0, 0};
      for (int q = plane_ptr[v]; q < plane_ptr[v + 1]; ++q) {
        const double *pl = planes + 4 * (size_t)q;
        for (int a = 0; a < 3; ++a) jl[a] = jl[a] + lambda[q] * pl[a];
      }
      for (int a = 0; a < 3; ++a) {
        double acc = 0.0;
        for (int k = row_ptr[v]; k < row_ptr[v + 1]; ++k) {
          if (cols[k] <= v) continue;
          const double *blk = vals + 9 * (size_t)k;
          const double *xc = x + 3 * (size_t)cols[k];
          for (int b = 0; b < 3; ++b) acc = acc + blk[3 * a + b] * xc[b];
        }
        rhs[3 * v + a] = (jl[a] - acc) + r[3 * v + a];
      }
    }
    for (int v = 0; v < nv; ++v) {
      double rv[3];
      for (int a = 0; a < 3; ++a) {
        double acc = rhs[3 * v + a];
        for (int k = row_ptr[v]; k < row_ptr[v + 1]; ++k) {
          if (cols[k] >= v) continue;
          const double *blk = vals + 9 * (size_t)k;
          const double *xc = x + 3 * (size_t)cols[k];
          for (int b = 0; b < 3; ++b) acc -= blk[3 * a + b] * xc[b];
        }
        rv[a] = acc;
      }
      mul3(&inv[9 * (size_t)v], rv, x + 3 * (size_t)v);
    }
    // residual = ||A x - r - J^T lambda|| (:390)
    double ss = 0.0;
    for (int v = 0; v < nv; ++v) {
      double jl[3] = {0, 0, 0};
      for (int q = plane_ptr[v]; q < plane_ptr[v + 1]; ++q) {
        const double *pl = planes + 4 * (size_t)q;
        for (int a = 0; a < 3; ++a) jl[a] = jl[a] + lambda[q] * pl[a];
      }
      for (int a = 0; a < 3; ++a) {
        double acc = 0.0;
        for (int k = row_ptr[v]; k < row_ptr[v + 1]; ++k) {
          const double *blk = vals + 9 * (size_t)k;
          const double *xc = x + 3 * (size_t)cols[k];
          for (int b = 0; b < 3; ++b) acc = acc + blk[3 * a + b] * xc[b];
        }
        const double t = (acc - r[3 * v + a]) - jl[a];
        ss = ss + t * t;
      }
    }
    st.residual = std::sqrt(ss);
    if (st.residual <= tol) {
      st.converged = 1;
      break;
    }
  }
  st.iterations = it;
  return st;
}

}  // namespace oracle
