// include/mprgp/MPRGPProjection.h -- projector and preconditioner types of the
// C++ façade, with the reference's names (src/MPRGPSolver/MPRGPProjection.h,
// MPRGPPrecondition.h).
//
// A projector here names the constraint set and carries the face (active
// set) that the GPU solve reports back; the per-iteration projector work runs
// inside the CUDA engine.  project() is also available on the host, because
// callers use it to make a start point feasible before solving
// (MprgpFemSolver.cpp:528).
#pragma once

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <vector>

#include "MPRGPUtility.h"

namespace MATH {

template <typename T>
struct ScalarUtil {
  static constexpr T scalar_max = (T)DBL_MAX;
  static constexpr T scalar_eps = (T)1e-9;  // src/CommonFile/MathBasic.cpp:9
};

// x >= L (MPRGPProjection.h:19-121).
template <typename T>
class LowerBoundProjector {
 public:
  explicit LowerBoundProjector(const Vec<T> &L) : _L(L), _face(L.size(), 0) {}
  const std::vector<char> &getFace() const { return _face; }
  std::vector<char> &face() { return _face; }
  const Vec<T> &lower() const { return _L; }
  void project(const Vec<T> &in, Vec<T> &out) const {
    out.resize(in.size());
    for (size_t i = 0; i < in.size(); ++i) out[i] = std::max(in[i], _L[i]);
  }

 private:
  const Vec<T> &_L;
  std::vector<char> _face;
};

// L <= x <= H (MPRGPProjection.h:124-238).
template <typename T>
class BoxBoundProjector {
 public:
  BoxBoundProjector(const Vec<T> &L, const Vec<T> &H) : _L(L), _H(H), _face(L.size(), 0) {}
  const std::vector<char> &getFace() const { return _face; }
  std::vector<char> &face() { return _face; }
  const Vec<T> &lower() const { return _L; }
  const Vec<T> &upper() const { return _H; }
  void project(const Vec<T> &in, Vec<T> &out) const {
    out.resize(in.size());
    for (size_t i = 0; i < in.size(); ++i) out[i] = std::min(std::max(in[i], _L[i]), _H[i]);
  }

 private:
  const Vec<T> &_L, &_H;
  std::vector<char> _face;
};

// J x >= c, common part (MPRGPProjection.h:241-317).
template <typename T>
class BaseGeneralConProjector {
 public:
  BaseGeneralConProjector(const SparseMatrix<T> &J, const Vec<T> &c)
      : J(J), c(c), face(J.rows(), 0) {}
  const std::vector<char> &getFace() const { return face; }
  std::vector<char> &faceRef() { return face; }
  const SparseMatrix<T> &getConMatrix() const { return J; }
  const Vec<T> &rhs() const { return c; }

 protected:
  const SparseMatrix<T> &J;
  const Vec<T> &c;
  std::vector<char> face;
};

// J J^T diagonal (MPRGPProjection.h:320-397).
template <typename T>
class DecoupledConProjector : public BaseGeneralConProjector<T> {
 public:
  DecoupledConProjector(const SparseMatrix<T> &J, const Vec<T> &JJt, const Vec<T> &c)
      : BaseGeneralConProjector<T>(J, c), JJt(JJt) {}
  // y = x + J^T max((c - J x) / JJt, 0)   (MPRGPProjection.h:333-348)
  void project(const Vec<T> &x, Vec<T> &y) const {
    y = x;
    const auto &ptr = this->J.outerIndex();
    const auto &idx = this->J.innerIndex();
    const auto &val = this->J.values();
    std::vector<T> lam(this->J.rows());
    for (int r = 0; r < this->J.rows(); ++r) {
      T jx = 0;
      for (int k = ptr[r]; k < ptr[r + 1]; ++k) jx += val[k] * x[idx[k]];
      lam[r] = std::max((this->c[r] - jx) / JJt[r], (T)0);
    }
    for (int r = 0; r < this->J.rows(); ++r)
      for (int k = ptr[r]; k < ptr[r + 1]; ++k) y[idx[k]] += val[k] * lam[r];
  }

 private:
  const Vec<T> &JJt;
};

// J J^T general, rows grouped per vertex (MPRGPProjection.h:400-520).  The
// projection onto each vertex's <= 3 half-spaces is solved exactly by
// enumerating active subsets (the QP is separable by vertex).
template <typename T>
class GeneralConProjector : public BaseGeneralConProjector<T> {
 public:
  GeneralConProjector(const SparseMatrix<T> &J, const Vec<T> &c)
      : BaseGeneralConProjector<T>(J, c) {}
  void project(const Vec<T> &x, Vec<T> &y) const {
    y = x;
    const auto &ptr = this->J.outerIndex();
    const auto &idx = this->J.innerIndex();
    const auto &val = this->J.values();
    // group rows by vertex (rows must touch one vertex's 3 columns)
    std::vector<std::vector<int>> by_vertex((x.size() + 2) / 3);
    for (int r = 0; r < this->J.rows(); ++r)
      if (ptr[r + 1] > ptr[r]) by_vertex[idx[ptr[r]] / 3].push_back(r);
    for (size_t v = 0; v < by_vertex.size(); ++v) {
      const auto &rows = by_vertex[v];
      const int k = (int)rows.size();
      if (k == 0 || k > 3) continue;
      T n[3][3] = {}, q[3] = {};
      for (int a = 0; a < k; ++a) {
        for (int p = ptr[rows[a]]; p < ptr[rows[a] + 1]; ++p) n[a][idx[p] - 3 * v] = val[p];
        q[a] = this->c[rows[a]] - (n[a][0] * x[3 * v] + n[a][1] * x[3 * v + 1] +
                                   (3 * v + 2 < x.size() ? n[a][2] * x[3 * v + 2] : 0));
      }
      T lam[3] = {};
      solve_vertex(n, q, k, lam);
      for (int a = 0; a < k; ++a)
        for (int d = 0; d < 3; ++d)
          if (3 * v + d < y.size()) y[3 * v + d] += n[a][d] * lam[a];
    }
  }

 private:
  // min 0.5 l^T G l - q^T l, l >= 0 (G = N N^T), by increasing support size.
  static void solve_vertex(const T n[3][3], const T q[3], int k, T lam[3]) {
    T G[3][3];
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b)
        G[a][b] = n[a][0] * n[b][0] + n[a][1] * n[b][1] + n[a][2] * n[b][2];
    T qmax = 1e-300;
    for (int a = 0; a < k; ++a) qmax = std::max(qmax, std::fabs(q[a]));
    const T tol = (T)1e-12 * qmax;
    for (int size = 0; size <= k; ++size)
      for (int mask = 0; mask < (1 << k); ++mask) {
        if (__builtin_popcount(mask) != size) continue;
        int S[3], s = 0;
        for (int a = 0; a < k; ++a)
          if (mask & (1 << a)) S[s++] = a;
        T t[3] = {};
        if (s == 1) {
          t[S[0]] = q[S[0]] / G[S[0]][S[0]];
        } else if (s == 2) {
          const int a = S[0], b = S[1];
          const T det = G[a][a] * G[b][b] - G[a][b] * G[b][a];
          if (!(det > 0)) continue;
          t[a] = (q[a] * G[b][b] - G[a][b] * q[b]) / det;
          t[b] = (G[a][a] * q[b] - G[b][a] * q[a]) / det;
        } else if (s == 3) {
          const T c00 = G[1][1] * G[2][2] - G[1][2] * G[2][1];
          const T c01 = G[1][2] * G[2][0] - G[1][0] * G[2][2];
          const T c02 = G[1][0] * G[2][1] - G[1][1] * G[2][0];
          const T det = G[0][0] * c00 + G[0][1] * c01 + G[0][2] * c02;
          if (!(det > 0)) continue;
          const T c10 = G[0][2] * G[2][1] - G[0][1] * G[2][2];
          const T c11 = G[0][0] * G[2][2] - G[0][2] * G[2][0];
          const T c12 = G[0][1] * G[2][0] - G[0][0] * G[2][1];
          const T c20 = G[0][1] * G[1][2] - G[0][2] * G[1][1];
          const T c21 = G[0][2] * G[1][0] - G[0][0] * G[1][2];
          const T c22 = G[0][0] * G[1][1] - G[0][1] * G[1][0];
          t[0] = (c00 * q[0] + c10 * q[1] + c20 * q[2]) / det;
          t[1] = (c01 * q[0] + c11 * q[1] + c21 * q[2]) / det;
          t[2] = (c02 * q[0] + c12 * q[1] + c22 * q[2]) / det;
        }
        T viol = 0;
        for (int a = 0; a < k; ++a) {
          if (mask & (1 << a)) {
            viol = std::max(viol, -t[a]);
          } else {
            T gr = -q[a];
            for (int b = 0; b < k; ++b) gr += G[a][b] * t[b];
            viol = std::max(viol, -gr);
          }
        }
        if (viol <= tol) {
          for (int a = 0; a < k; ++a) lam[a] = std::max(t[a], (T)0);
          return;
        }
      }
  }
};

// Preconditioner selectors (MPRGPPrecondition.h).  The preconditioner runs
// inside the engine; these types only select it for MPRGP / MPRGPMonotonic.
template <typename T, typename MAT, bool NO_PRECOND = false>
struct DiagonalInFacePreconSolver {
  template <typename... Args>
  explicit DiagonalInFacePreconSolver(Args &&...) {}
  static constexpr int engine_precond = NO_PRECOND ? 1 : 2;
};
template <typename T, typename MAT, bool NO_PRECOND = false>
struct DiagonalDecouplePreconSolver {
  template <typename... Args>
  explicit DiagonalDecouplePreconSolver(Args &&...) {}
  static constexpr int engine_precond = NO_PRECOND ? 1 : 3;
};
template <typename T, typename MAT>
struct InFaceNoPreconSolver {
  template <typename... Args>
  explicit InFaceNoPreconSolver(Args &&...) {}
  static constexpr int engine_precond = 1;
};

}  // namespace MATH
