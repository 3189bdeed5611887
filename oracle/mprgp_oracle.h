// oracle/mprgp_oracle.h -- CPU restatement of the reference MPRGP solver.
//
// TEST INFRASTRUCTURE ONLY.  This header is the parity oracle for the GPU
// solver: only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline /
// --impl reference leg may load it.  The product path (mprgp_gb300/) never
// links, imports or calls anything under oracle/.
//
// It restates, line by line, the control flow and arithmetic of
//   src/MPRGPSolver/MPRGPSolver.h      (MPRGPBase, MPRGP, MPRGPMonotonic,
//                                        FixedSparseMatrix, the solve façades)
//   src/MPRGPSolver/MPRGPProjection.h  (Lower/Box/Decoupled/General projectors)
//   src/MPRGPSolver/MPRGPPrecondition.h(InFace / DiagonalInFace / DiagonalDecouple)
//   src/MPRGPSolver/MPRGPUtility.h     (MASK_FACE, COUNT_CONSTRAINTS, convert,
//                                        getDiagonal)
// over plain CSR matrices and std::vector<double> (Eigen is not available).
//
// Deliberate, documented differences from the reference:
//  * specRad's start vector: the reference calls Eigen's setRandom()
//    (std::rand, unseeded).  Here it is seeded_uniform(seed, i), a
//    splitmix64 hash mapped to [-1, 1); the GPU path uses the same formula.
//  * GeneralConProjector: the reference solves one dense QP over ALL
//    constraint rows with QuadProg++ (MPRGPProjection.h:412-430, 450-467) and
//    a sparse LLT (:431-449).  The QP is block-separable: rows that share no
//    column are independent.  This restatement splits the rows into those
//    blocks once and solves each block exactly (active-set enumeration for the
//    projection / BETA QPs, Cholesky for PHI).  The answer is the same QP
//    solution; tests cross-check it against QuadProg++ compiled from the
//    reference's own sources.
//
// Parity status: the reference's MPRGP path cannot be compiled here (it needs
// Eigen3 and Boost, absent from the image), and its own tests hold no golden
// vectors for this path (MPRGPTest.cpp asserts properties; its qp33.b fixture
// is missing).  The oracle is pinned by (a) those properties, (b) QuadProg++
// built from src/MPRGPSolver/SimpleQP/ solving the same QPs, (c) KKT checks.
#pragma once

#include <algorithm>
#include <array>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

namespace oracle {

using Vec = std::vector<double>;

// MPRGPUtility.h:72-83 declares ScalarUtil; the values come from
// src/CommonFile/MathBasic.cpp:8-9 and test_case/main.cpp:12-13.
struct ScalarUtil {
  static constexpr double scalar_max = DBL_MAX;
  static constexpr double scalar_eps = 1e-9;
};

// ---------------------------------------------------------------- vectors --
// Thread count of the optional OpenMP build (the reference's serial path is
// 1 thread; OMP_PARALLEL_FOR_ is empty in MPRGPUtility.h:64).
inline int &omp_threads() {
  static int n = 1;
  return n;
}

inline double dot(const Vec &a, const Vec &b) {
  double s = 0.0;
  const long long n = (long long)a.size();
#ifdef _OPENMP
#pragma omp parallel for reduction(+ : s) num_threads(omp_threads()) if (omp_threads() > 1)
#endif
  for (long long i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}
inline double norm(const Vec &a) { return std::sqrt(dot(a, a)); }

// Seeded replacement for Eigen's setRandom(): uniform in [-1, 1).
inline uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  uint64_t z = x;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
inline double seeded_uniform(uint64_t seed, uint64_t i) {
  const uint64_t h = splitmix64(seed * 0x9E3779B97F4A7C15ull + i);
  return 2.0 * ((double)(h >> 11) * 0x1.0p-53) - 1.0;
}

// ------------------------------------------------------------- CSR matrix --
struct Csr {
  int rows = 0, cols = 0;
  std::vector<int> ptr, idx;
  std::vector<double> val;
  Csr() { ptr.assign(1, 0); }
  int nonZeros() const { return (int)idx.size(); }
  void multiply(const Vec &x, Vec &y) const {  // y = M x
    y.assign(rows, 0.0);
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(omp_threads()) if (omp_threads() > 1)
#endif
    for (int r = 0; r < rows; ++r) {
      double s = 0.0;
      for (int k = ptr[r]; k < ptr[r + 1]; ++k) s += val[k] * x[idx[k]];
      y[r] = s;
    }
  }
  void multiplyT(const Vec &x, Vec &y) const {  // y = M^T x
    y.assign(cols, 0.0);
    for (int r = 0; r < rows; ++r)
      for (int k = ptr[r]; k < ptr[r + 1]; ++k) y[idx[k]] += val[k] * x[r];
  }
  // getDiagonal (MPRGPUtility.h:503-515); missing diagonal entries are 0.
  Vec diagonal() const {
    Vec d(std::min(rows, cols), 0.0);
    for (int r = 0; r < (int)d.size(); ++r)
      for (int k = ptr[r]; k < ptr[r + 1]; ++k)
        if (idx[k] == r) { d[r] = val[k]; break; }
    return d;
  }
  // diag(J J^T) and diag(J D J^T) for a diagonal D.
  Vec rowNorm2(const Vec *D = nullptr) const {
    Vec d(rows, 0.0);
    for (int r = 0; r < rows; ++r)
      for (int k = ptr[r]; k < ptr[r + 1]; ++k)
        d[r] += val[k] * val[k] * (D ? (*D)[idx[k]] : 1.0);
    return d;
  }
};

// --------------------------------------------------------------- utility --
// MASK_FACE (MPRGPUtility.h:85-96)
inline void MASK_FACE(const Vec &in, Vec &out, const std::vector<char> &face) {
  out.resize(in.size());
  for (size_t i = 0; i < in.size(); ++i) out[i] = (0 != face[i]) ? 0.0 : in[i];
}
// COUNT_CONSTRAINTS (MPRGPUtility.h:98-106): note it sums the face codes.
inline int COUNT_CONSTRAINTS(const std::vector<char> &face) {
  int c = 0;
  for (char f : face) c += (int)f;
  return c;
}

// Small dense helpers for the block-separable GeneralConProjector.
// Cholesky solve of an SPD k x k system (row-major G), in place on rhs.
inline bool chol_solve(std::vector<double> G, int k, std::vector<double> &rhs) {
  for (int j = 0; j < k; ++j) {
    double d = G[j * k + j];
    for (int p = 0; p < j; ++p) d -= G[j * k + p] * G[j * k + p];
    if (!(d > 0.0)) return false;
    d = std::sqrt(d);
    G[j * k + j] = d;
    for (int i = j + 1; i < k; ++i) {
      double s = G[i * k + j];
      for (int p = 0; p < j; ++p) s -= G[i * k + p] * G[j * k + p];
      G[i * k + j] = s / d;
    }
  }
  for (int i = 0; i < k; ++i) {
    double s = rhs[i];
    for (int p = 0; p < i; ++p) s -= G[i * k + p] * rhs[p];
    rhs[i] = s / G[i * k + i];
  }
  for (int i = k - 1; i >= 0; --i) {
    double s = rhs[i];
    for (int p = i + 1; p < k; ++p) s -= G[p * k + i] * rhs[p];
    rhs[i] = s / G[i * k + i];
  }
  return true;
}

// min 0.5 l^T G l - q^T l  s.t. l >= 0, for a small SPD G (k <= 12), by
// enumerating the support set and keeping the one that satisfies KKT.  This is
// the per-block restatement of solveQP(G, q, I, 0, l) (SimpleQP.h:17-48).
inline void nonneg_qp(const std::vector<double> &G, const std::vector<double> &q,
                      int k, std::vector<double> &lam) {
  lam.assign(k, 0.0);
  if (k == 0) return;
  double scale = 1e-300;
  for (int i = 0; i < k; ++i) scale = std::max(scale, std::fabs(q[i]));
  for (int i = 0; i < k * k; ++i) scale = std::max(scale, std::fabs(G[i]) * 1e-300);
  const double tol = 1e-12 * scale;
  double best_viol = DBL_MAX;
  std::vector<double> best(k, 0.0), trial(k), sub, rhs;
  std::vector<int> S;
  const int nsub = 1 << k;
  // Enumerate by increasing support size so the smallest valid support wins.
  for (int size = 0; size <= k; ++size) {
    for (int mask = 0; mask < nsub; ++mask) {
      if (__builtin_popcount((unsigned)mask) != size) continue;
      S.clear();
      for (int i = 0; i < k; ++i)
        if (mask & (1 << i)) S.push_back(i);
      const int s = (int)S.size();
      std::fill(trial.begin(), trial.end(), 0.0);
      if (s > 0) {
        sub.assign(s * s, 0.0);
        rhs.assign(s, 0.0);
        for (int a = 0; a < s; ++a) {
          rhs[a] = q[S[a]];
          for (int b = 0; b < s; ++b) sub[a * s + b] = G[S[a] * k + S[b]];
        }
        if (!chol_solve(sub, s, rhs)) continue;
        for (int a = 0; a < s; ++a) trial[S[a]] = rhs[a];
      }
      double viol = 0.0;
      for (int i = 0; i < k; ++i) {
        if (mask & (1 << i)) {
          viol = std::max(viol, -trial[i]);
        } else {
          double gr = -q[i];
          for (int j = 0; j < k; ++j) gr += G[i * k + j] * trial[j];
          viol = std::max(viol, -gr);
        }
      }
      if (viol <= tol) {
        for (int i = 0; i < k; ++i) lam[i] = std::max(trial[i], 0.0);
        return;
      }
      if (viol < best_viol) { best_viol = viol; best = trial; }
    }
  }
  for (int i = 0; i < k; ++i) lam[i] = std::max(best[i], 0.0);
}

// ============================================================ projectors ==
// LowerBoundProjector (MPRGPProjection.h:19-121): x >= L.
class LowerBoundProjector {
 public:
  explicit LowerBoundProjector(const Vec &L) : _L(L), _face(L.size(), 0) {}
  const std::vector<char> &getFace() const { return _face; }
  double stepLimit(const Vec &X, const Vec &D, double = ScalarUtil::scalar_max) const {
    double tmp = ScalarUtil::scalar_max;  // :34-53
    for (size_t i = 0; i < X.size(); ++i)
      if (D[i] > ScalarUtil::scalar_eps && X[i] > _L[i])
        tmp = std::min(tmp, (X[i] - _L[i]) / D[i]);
    return tmp;
  }
  void project(const Vec &in, Vec &out) const {  // :56-62
    out.resize(_L.size());
    for (size_t i = 0; i < in.size(); ++i) out[i] = std::max(in[i], _L[i]);
  }
  void PHI(const Vec &in, Vec &out) { MASK_FACE(in, out, _face); }
  void BETA(const Vec &in, Vec &out, const Vec &) {  // :66-77
    out.resize(in.size());
    for (size_t i = 0; i < in.size(); ++i)
      out[i] = (0 == _face[i]) ? 0.0 : std::min(in[i], 0.0);
  }
  void DECIDE_FACE(const Vec &x) {  // :78-90
    _face.assign(x.size(), 0);
    for (size_t i = 0; i < x.size(); ++i)
      if (std::fabs(x[i] - _L[i]) < ScalarUtil::scalar_eps) _face[i] = 2;
  }
  double PHITPHI(const Vec &x, double alphaBar, const Vec &phi) {  // :91-106
    double s = 0.0;
    for (size_t i = 0; i < x.size(); ++i) {
      double t = 0.0;
      if (phi[i] > 0.0 && x[i] > _L[i]) t = std::min((x[i] - _L[i]) / alphaBar, phi[i]);
      s += t * phi[i];
    }
    return s;
  }
  bool isFeasible(const Vec &x) const {  // :108-116
    for (size_t i = 0; i < x.size(); ++i)
      if (x[i] < _L[i] - ScalarUtil::scalar_eps) return false;
    return true;
  }

 private:
  const Vec &_L;
  std::vector<char> _face;
};

// BoxBoundProjector (MPRGPProjection.h:124-238): L <= x <= H.
class BoxBoundProjector {
 public:
  BoxBoundProjector(const Vec &L, const Vec &H) : _L(L), _H(H), _face(L.size(), 0) {}
  const std::vector<char> &getFace() const { return _face; }
  double stepLimit(const Vec &X, const Vec &D, double = ScalarUtil::scalar_max) const {
    double tmp = ScalarUtil::scalar_max;  // :139-162
    for (size_t i = 0; i < X.size(); ++i) {
      if (D[i] > ScalarUtil::scalar_eps && X[i] > _L[i])
        tmp = std::min(tmp, (X[i] - _L[i]) / D[i]);
      else if (D[i] < -ScalarUtil::scalar_eps && X[i] < _H[i])
        tmp = std::min(tmp, (X[i] - _H[i]) / D[i]);
    }
    return tmp;
  }
  void project(const Vec &in, Vec &out) const {  // :163-169
    out.resize(_L.size());
    for (size_t i = 0; i < in.size(); ++i) out[i] = std::min(std::max(in[i], _L[i]), _H[i]);
  }
  void PHI(const Vec &in, Vec &out) { MASK_FACE(in, out, _face); }
  void BETA(const Vec &in, Vec &out, const Vec &) {  // :173-186
    out.resize(in.size());
    for (size_t i = 0; i < in.size(); ++i) {
      if (_face[i] == 0) out[i] = 0.0;
      else if (_face[i] == 1) out[i] = std::max(in[i], 0.0);
      else out[i] = std::min(in[i], 0.0);
    }
  }
  void DECIDE_FACE(const Vec &x) {  // :187-201
    _face.assign(x.size(), 0);
    for (size_t i = 0; i < x.size(); ++i) {
      if (std::fabs(x[i] - _L[i]) < ScalarUtil::scalar_eps) _face[i] = 2;
      else if (std::fabs(x[i] - _H[i]) < ScalarUtil::scalar_eps) _face[i] = 1;
    }
  }
  double PHITPHI(const Vec &x, double alphaBar, const Vec &phi) {  // :202-221
    double s = 0.0;
    for (size_t i = 0; i < x.size(); ++i) {
      double t = 0.0;
      if (phi[i] > 0.0 && x[i] > _L[i]) t = std::min((x[i] - _L[i]) / alphaBar, phi[i]);
      else if (phi[i] < 0.0 && x[i] < _H[i]) t = std::max((x[i] - _H[i]) / alphaBar, phi[i]);
      s += t * phi[i];
    }
    return s;
  }
  bool isFeasible(const Vec &x) const {  // :223-232
    for (size_t i = 0; i < x.size(); ++i)
      if (x[i] < _L[i] - ScalarUtil::scalar_eps || x[i] > _H[i] + ScalarUtil::scalar_eps)
        return false;
    return true;
  }

 private:
  const Vec &_L, &_H;
  std::vector<char> _face;
};

// BaseGeneralConProjector (MPRGPProjection.h:241-317): J x >= c.
class BaseGeneralConProjector {
 public:
  BaseGeneralConProjector(const Csr &J, const Vec &c) : J(J), c(c), face(J.rows, 0) {}
  const std::vector<char> &getFace() const { return face; }
  const Csr &getConMatrix() const { return J; }
  double stepLimit(const Vec &X, const Vec &D, double alpha_cg = ScalarUtil::scalar_max) const {
    double alpha = (alpha_cg == ScalarUtil::scalar_max) ? alpha_cg
                                                        : (alpha_cg + ScalarUtil::scalar_eps);
    Vec Jx, Jd;  // :263-282
    J.multiply(X, Jx);
    J.multiply(D, Jd);
    for (int i = 0; i < J.rows; ++i)
      if (Jd[i] > ScalarUtil::scalar_eps && Jx[i] > c[i])
        alpha = std::min(alpha, (Jx[i] - c[i]) / Jd[i]);
    return alpha;
  }
  void DECIDE_FACE(const Vec &x) {  // :283-297
    face.assign(c.size(), 0);
    Vec Jx;
    J.multiply(x, Jx);
    num_active_cons = 0;
    for (int i = 0; i < (int)c.size(); ++i)
      if (std::fabs(Jx[i] - c[i]) < ScalarUtil::scalar_eps) { face[i] = 1; ++num_active_cons; }
  }
  bool isFeasible(const Vec &x) const {  // :298-310
    Vec Jx;
    J.multiply(x, Jx);
    for (int i = 0; i < (int)c.size(); ++i)
      if (Jx[i] < c[i] - ScalarUtil::scalar_eps) return false;
    return true;
  }

 protected:
  const Csr &J;
  const Vec &c;
  std::vector<char> face;
  int num_active_cons = 0;
};

// DecoupledConProjector (MPRGPProjection.h:320-397): J J^T diagonal.
class DecoupledConProjector : public BaseGeneralConProjector {
 public:
  DecoupledConProjector(const Csr &J, const Vec &JJt, const Vec &c)
      : BaseGeneralConProjector(J, c), JJt(JJt) {}
  void project(const Vec &x, Vec &y) const {  // :333-348
    if (J.rows == 0) { y = x; return; }
    Vec lambda;
    J.multiply(x, lambda);
    for (int i = 0; i < (int)lambda.size(); ++i)
      lambda[i] = std::max((c[i] - lambda[i]) / JJt[i], 0.0);
    Vec t;
    J.multiplyT(lambda, t);
    y.resize(x.size());
    for (size_t i = 0; i < x.size(); ++i) y[i] = x[i] + t[i];
  }
  void PHI(const Vec &g, Vec &phi) const {  // :349-367
    if (num_active_cons == 0) { phi = g; return; }
    Vec lambda;
    J.multiply(g, lambda);
    for (size_t i = 0; i < face.size(); ++i)
      lambda[i] = (0 == face[i]) ? 0.0 : -lambda[i] / JJt[i];
    Vec t;
    J.multiplyT(lambda, t);
    phi.resize(g.size());
    for (size_t i = 0; i < g.size(); ++i) phi[i] = g[i] + t[i];
  }
  void BETA(const Vec &g, Vec &beta, const Vec &phi) const {  // :368-383
    beta.resize(g.size());
    for (size_t i = 0; i < g.size(); ++i) beta[i] = g[i] - phi[i];
    if (num_active_cons == 0) return;
    Vec lambda;
    J.multiply(beta, lambda);
    // Rows with face 0 keep lambda = (J beta)_i, as the reference does.
    for (size_t i = 0; i < face.size(); ++i)
      if (0 != face[i]) lambda[i] = std::max(0.0, lambda[i] / JJt[i]);
    Vec t;
    J.multiplyT(lambda, t);
    for (size_t i = 0; i < g.size(); ++i) beta[i] -= t[i];
  }
  double PHITPHI(const Vec &x, double alpha_bar, const Vec &phi) const {  // :384-393
    Vec xap(x.size()), px;
    for (size_t i = 0; i < x.size(); ++i) xap[i] = x[i] - alpha_bar * phi[i];
    project(xap, px);
    double s = 0.0;
    for (size_t i = 0; i < x.size(); ++i) s += (x[i] - px[i]) * phi[i];
    const double phitphi = s * (1.0 / alpha_bar);
    return phitphi > 0.0 ? phitphi : 0.0;
  }

 private:
  const Vec &JJt;
};

// GeneralConProjector (MPRGPProjection.h:400-520), block-separable form.
class GeneralConProjector : public BaseGeneralConProjector {
 public:
  GeneralConProjector(const Csr &J, const Vec &c) : BaseGeneralConProjector(J, c) {
    buildBlocks();
  }
  // project (:412-430): y = x + J^T l, l = argmin 0.5 l^T JJ^T l - (c - Jx)^T l, l >= 0.
  void project(const Vec &x, Vec &y) const {
    y = x;
    if (J.rows == 0) return;
    Vec Jx;
    J.multiply(x, Jx);
    std::vector<double> G, q, lam;
    for (const auto &blk : blocks) {
      const int k = (int)blk.size();
      gram(blk, G);
      q.resize(k);
      for (int a = 0; a < k; ++a) q[a] = c[blk[a]] - Jx[blk[a]];
      nonneg_qp(G, q, k, lam);
      for (int a = 0; a < k; ++a) addRowT(blk[a], lam[a], y);
    }
  }
  // PHI (:431-449): phi = g + J_a^T l, (J_a J_a^T) l = -J_a g.
  void PHI(const Vec &g, Vec &phi) const {
    phi = g;
    std::vector<int> act;
    std::vector<double> G, rhs;
    for (const auto &blk : blocks) {
      act.clear();
      for (int r : blk)
        if (1 == face[r]) act.push_back(r);
      if (act.empty()) continue;
      const int k = (int)act.size();
      gram(act, G);
      rhs.resize(k);
      for (int a = 0; a < k; ++a) rhs[a] = -rowDot(act[a], g);
      if (!chol_solve(G, k, rhs)) continue;  // reference: ERROR_LOG, no update
      for (int a = 0; a < k; ++a) addRowT(act[a], rhs[a], phi);
    }
  }
  // BETA (:450-467): beta = gp - J_a^T l, l = argmin 0.5 l^T G l - (J_a gp)^T l, l >= 0.
  void BETA(const Vec &g, Vec &beta, const Vec &phi) const {
    beta.resize(g.size());
    for (size_t i = 0; i < g.size(); ++i) beta[i] = g[i] - phi[i];
    std::vector<int> act;
    std::vector<double> G, q, lam;
    const Vec gp = beta;
    for (const auto &blk : blocks) {
      act.clear();
      for (int r : blk)
        if (1 == face[r]) act.push_back(r);
      if (act.empty()) continue;
      const int k = (int)act.size();
      gram(act, G);
      q.resize(k);
      for (int a = 0; a < k; ++a) q[a] = rowDot(act[a], gp);
      nonneg_qp(G, q, k, lam);
      for (int a = 0; a < k; ++a) addRowT(act[a], -lam[a], beta);
    }
  }
  double PHITPHI(const Vec &x, double alpha_bar, const Vec &phi) const {  // :468-478
    Vec xap(x.size()), px;
    for (size_t i = 0; i < x.size(); ++i) xap[i] = x[i] - alpha_bar * phi[i];
    project(xap, px);
    double s = 0.0;
    for (size_t i = 0; i < x.size(); ++i) s += (x[i] - px[i]) * phi[i];
    const double phitphi = s * (1.0 / alpha_bar);
    return phitphi > 0.0 ? phitphi : 0.0;
  }

 private:
  std::vector<std::vector<int>> blocks;  // rows grouped by shared columns
  double rowDot(int r, const Vec &v) const {
    double s = 0.0;
    for (int k = J.ptr[r]; k < J.ptr[r + 1]; ++k) s += J.val[k] * v[J.idx[k]];
    return s;
  }
  void addRowT(int r, double s, Vec &v) const {
    for (int k = J.ptr[r]; k < J.ptr[r + 1]; ++k) v[J.idx[k]] += J.val[k] * s;
  }
  double rowRow(int r1, int r2) const {
    double s = 0.0;
    for (int a = J.ptr[r1]; a < J.ptr[r1 + 1]; ++a)
      for (int b = J.ptr[r2]; b < J.ptr[r2 + 1]; ++b)
        if (J.idx[a] == J.idx[b]) s += J.val[a] * J.val[b];
    return s;
  }
  void gram(const std::vector<int> &rows, std::vector<double> &G) const {
    const int k = (int)rows.size();
    G.assign(k * k, 0.0);
    for (int a = 0; a < k; ++a)
      for (int b = 0; b < k; ++b) G[a * k + b] = rowRow(rows[a], rows[b]);
  }
  void buildBlocks() {  // union-find over rows that share a column
    const int m = J.rows;
    std::vector<int> parent(m);
    std::iota(parent.begin(), parent.end(), 0);
    auto find = [&](int a) {
      while (parent[a] != a) a = parent[a] = parent[parent[a]];
      return a;
    };
    std::vector<int> owner(J.cols, -1);
    for (int r = 0; r < m; ++r)
      for (int k = J.ptr[r]; k < J.ptr[r + 1]; ++k) {
        const int col = J.idx[k];
        if (owner[col] < 0) owner[col] = r;
        else parent[find(r)] = find(owner[col]);
      }
    std::vector<int> bid(m, -1);
    for (int r = 0; r < m; ++r) {
      const int root = find(r);
      if (bid[root] < 0) { bid[root] = (int)blocks.size(); blocks.emplace_back(); }
      blocks[bid[root]].push_back(r);
    }
  }
};

// ======================================================= preconditioners ==
// InFaceNoPreconSolver (MPRGPPrecondition.h:19-33)
class InFaceNoPreconSolver {
 public:
  explicit InFaceNoPreconSolver(const std::vector<char> &face) : _face(face) {}
  int solve(const Vec &rhs, Vec &result, const Vec &) const {
    MASK_FACE(rhs, result, _face);
    return 0;
  }

 private:
  const std::vector<char> &_face;
};

// DiagonalInFacePreconSolver (MPRGPPrecondition.h:36-69)
template <typename MAT, bool NO_PRECOND = false>
class DiagonalInFacePreconSolver {
 public:
  DiagonalInFacePreconSolver(const MAT &M, const std::vector<char> &face) : face(face) {
    invert_diag.resize(M.rows());
    if (!NO_PRECOND)
      for (int i = 0; i < (int)invert_diag.size(); ++i) invert_diag[i] = 1.0 / M.diag(i);
  }
  int solve(const Vec &g, Vec &z, const Vec &phi) const {
    (void)g;
    if (!NO_PRECOND) {
      z.resize(phi.size());
      for (size_t i = 0; i < z.size(); ++i) z[i] = phi[i] * invert_diag[i];
    } else {
      z = phi;
    }
    return 0;
  }

 protected:
  Vec invert_diag;
  const std::vector<char> &face;
};

// DiagonalDecouplePreconSolver (MPRGPPrecondition.h:72-110)
template <typename MAT, bool NO_PRECOND = false>
class DiagonalDecouplePreconSolver : public DiagonalInFacePreconSolver<MAT, NO_PRECOND> {
  using Base = DiagonalInFacePreconSolver<MAT, NO_PRECOND>;

 public:
  DiagonalDecouplePreconSolver(const MAT &M, const std::vector<char> &face, const Csr &J)
      : Base(M, face), J(J) {
    if (!NO_PRECOND && J.rows > 0) {
      has_j = true;
      invert_JMinvJt = J.rowNorm2(&this->invert_diag);  // diag(J D^-1 J^T)
      for (double &v : invert_JMinvJt) v = 1.0 / v;
    }
  }
  int solve(const Vec &g, Vec &z, const Vec &phi) const {
    if (!NO_PRECOND && has_j) {
      const Vec &Dinv = this->invert_diag;
      Vec Dg(g.size());
      for (size_t i = 0; i < g.size(); ++i) Dg[i] = Dinv[i] * g[i];
      Vec lambda;  // invert_JMinvJt .* (J D^-1 g)
      J.multiply(Dg, lambda);
      for (size_t i = 0; i < lambda.size(); ++i)
        lambda[i] = (0 == this->face[i]) ? 0.0 : invert_JMinvJt[i] * lambda[i];
      Vec t;  // (J D^-1)^T lambda = D^-1 J^T lambda
      J.multiplyT(lambda, t);
      z.resize(g.size());
      for (size_t i = 0; i < g.size(); ++i) z[i] = Dg[i] - Dinv[i] * t[i];
    } else {
      z = phi;
    }
    return 0;
  }

 private:
  const Csr &J;
  bool has_j = false;
  Vec invert_JMinvJt;
};

// ============================================================ the matrix ==
// FixedSparseMatrix (MPRGPSolver.h:459-500)
class FixedSparseMatrix {
 public:
  explicit FixedSparseMatrix(const Csr &M) : A(M), diag_A(M.diagonal()) {}
  void multiply(const Vec &x, Vec &y) const { A.multiply(x, y); }
  double funcValue(const Vec &x, const Vec &b) const {  // 1/2 x^T A x - x^T b
    Vec Ax;
    A.multiply(x, Ax);
    return 0.5 * dot(x, Ax) - dot(x, b);
  }
  int rows() const { return A.rows; }
  double diag(int i) const { return diag_A[i]; }
  const Csr &getMatrix() const { return A; }

 private:
  const Csr &A;
  Vec diag_A;
};

// Step trace (test diagnostics): {event, iteration, residual, value}.
// event 1 CG commit (value f(P(y))-f(x)), 2 CG exit (same), 3 expansion,
// 4 proportioning, 5 loop top (value = proportional).
using Trace = std::vector<std::array<double, 4>>;

struct SolveStats {
  int code = -1, iterations = 0, num_cg = 0, num_exp = 0, num_prop = 0, power_iters = 0;
  int spmv = 0;
  double residual = 0.0, alpha_bar = 0.0, spec_rad = 0.0;
};

// ================================================================= MPRGP ==
// MPRGPBase (MPRGPSolver.h:15-342)
template <typename MAT, typename PROJ, typename PRECOND>
class MPRGPBase {
 public:
  MPRGPBase(const MAT &A, const Vec &B, PRECOND &precond, PROJ &projector, int max_it,
            double tol, Vec *ev, uint64_t seed)
      : A(A), B(B), precond(precond), projector(projector) {
    max_iterations = max_it;  // setParameters (:34-39)
    tolerance_factor = tol < 1e-30 ? 1e-30 : tol;
    gamma = 1.0;
    spec_rad = specRad(A, ev, tol, seed, &power_iters, &spmv);
    alpha_bar = 2.0 / spec_rad;
  }
  // specRad (:42-79) with a seeded start vector.
  static double specRad(const MAT &G, Vec *ev, double eps, uint64_t seed, int *iters_out,
                        int *spmv_count) {
    const int n = G.rows();
    Vec tmp, tmpOut(n);
    if (ev != nullptr && (int)ev->size() == n) {
      tmp = *ev;
    } else {
      tmp.resize(n);
      for (int i = 0; i < n; ++i) tmp[i] = seeded_uniform(seed, (uint64_t)i);
      const double nr = norm(tmp);
      for (double &v : tmp) v /= nr;
    }
    double normTmpOut = 1.0;
    int iter = 0;
    for (; iter <= 1000; ++iter) {
      G.multiply(tmp, tmpOut);
      ++*spmv_count;
      normTmpOut = norm(tmpOut);
      if (normTmpOut < ScalarUtil::scalar_eps) {
        if (ev) *ev = tmp;
        normTmpOut = ScalarUtil::scalar_eps;
        break;
      }
      for (double &v : tmpOut) v /= normTmpOut;
      double d2 = 0.0;
      for (int i = 0; i < n; ++i) d2 += (tmpOut[i] - tmp[i]) * (tmpOut[i] - tmp[i]);
      if (std::sqrt(d2) <= eps) {
        if (ev) *ev = tmp;
        break;
      }
      tmp = tmpOut;
    }
    if (iters_out) *iters_out = iter;
    return normTmpOut;
  }
  SolveStats stats() const {
    SolveStats s;
    s.code = result_code;
    s.iterations = (int)iterations_out;
    s.num_cg = num_cg;
    s.num_exp = num_exp;
    s.num_prop = numprop;
    s.power_iters = power_iters;
    s.residual = residual_out;
    s.alpha_bar = alpha_bar;
    s.spec_rad = spec_rad;
    s.spmv = spmv;
    return s;
  }

 protected:
  void mul(const Vec &x, Vec &y) { A.multiply(x, y); ++spmv; }
  double fval(const Vec &x) { ++spmv; return A.funcValue(x, B); }
  void gradient(const Vec &x) {  // g = A x - B
    mul(x, g);
    for (size_t i = 0; i < g.size(); ++i) g[i] -= B[i];
  }
  void initialize(const Vec &result) {  // :148-162
    gradient(result);
    g_exact = true;
    projector.DECIDE_FACE(result);
    projector.PHI(g, phi);
    precond.solve(g, z, phi);
    p = z;
    result_code = -1;
    num_cg = num_exp = numprop = iteration = 0;
  }
  double computeGradients(const Vec &gg, bool comp_phi = true) {  // :163-173
    if (comp_phi) projector.PHI(gg, phi);
    projector.BETA(gg, beta, phi);
    gp.resize(phi.size());
    for (size_t i = 0; i < phi.size(); ++i) gp[i] = phi[i] + beta[i];
    return norm(gp);
  }
  bool proportional(const Vec &result) {  // :174-181
    const double left = dot(beta, beta);
    const double right = gamma * gamma * projector.PHITPHI(result, alpha_bar, phi);
    return left <= right;
  }
  void CGStep(const Vec &AP, double alpha_cg, Vec &result) {  // :182-195
    ++num_cg;
    for (size_t i = 0; i < result.size(); ++i) {
      result[i] -= alpha_cg * p[i];
      g[i] -= alpha_cg * AP[i];
    }
    projector.PHI(g, phi);
    precond.solve(g, z, phi);
    const double b = dot(z, AP) / dot(p, AP);
    for (size_t i = 0; i < p.size(); ++i) p[i] = z[i] - b * p[i];
  }
  void ExpStep(const Vec &AP, double alpha_f, Vec &result) {  // :196-218
    ++num_exp;
    Vec &xTmp = beta;
    xTmp.resize(result.size());
    for (size_t i = 0; i < result.size(); ++i) {
      xTmp[i] = result[i] - alpha_f * p[i];
      g[i] -= alpha_f * AP[i];
    }
    projector.DECIDE_FACE(xTmp);
    projector.PHI(g, phi);
    for (size_t i = 0; i < xTmp.size(); ++i) xTmp[i] -= alpha_bar * phi[i];
    projector.project(xTmp, result);
    gradient(result);
    projector.DECIDE_FACE(result);
    projector.PHI(g, phi);
    precond.solve(g, z, phi);
    p = z;
  }
  void PropStep(Vec &result) {  // :219-243
    ++numprop;
    const Vec D = beta;
    Vec &AD = gp;
    mul(D, AD);
    const double ddad = dot(D, AD);
    const double alpha_cg = dot(g, D) / ddad;
    for (size_t i = 0; i < result.size(); ++i) result[i] -= alpha_cg * D[i];
    Vec &xTmp = beta;
    xTmp = result;
    projector.project(xTmp, result);
    // The recursive update below is A x - B in exact arithmetic only when the
    // projection moved nothing.
    g_exact = (xTmp == result);
    for (size_t i = 0; i < g.size(); ++i) g[i] -= alpha_cg * AD[i];
    projector.DECIDE_FACE(result);
    projector.PHI(g, phi);
    precond.solve(g, z, phi);
    p = z;
  }
  double projectFunValue(const Vec &x) {  // :245-249
    projector.project(x, tempx);
    return fval(tempx);
  }
  void ExpMonotonicStep(Vec &result) {  // :250-271
    ++num_exp;
    projector.project(result, y);
    gradient(y);
    projector.DECIDE_FACE(y);
    projector.PHI(g, phi);
    for (size_t i = 0; i < y.size(); ++i) y[i] -= alpha_bar * phi[i];
    projector.project(y, result);
    gradient(result);
    g_exact = true;
    projector.DECIDE_FACE(result);
    projector.PHI(g, phi);
    precond.solve(g, z, phi);
    p = z;
  }
  // f(P(y)) - f(x) for y = x - alpha p, from scalars (the scalar_test switch):
  //   f(y) - f(x)    = -alpha p.(A x - B) + alpha^2/2 p^T A p,
  //   f(P(y)) - f(y) = d.(A y - B) + d^T A d / 2,   d = P(y) - y,
  // where A x - B = g + e (e = 0 unless g is a recursive update that left
  // A x - B, see g_exact) and A y - B = g - alpha A p + e.  Writes y.
  // Returns f(y) - f(x) and sets corr = f(P(y)) - f(y).
  double scalar_decrease(const Vec &result, double alpha, double pd, const Vec &AP, const Vec *e,
                         double &corr) {
    const size_t n = result.size();
    y.resize(n);
    for (size_t i = 0; i < n; ++i) y[i] = result[i] - alpha * p[i];
    double pg = dot(p, g);
    if (e) pg += dot(p, *e);
    const double dfy = -alpha * pg + 0.5 * alpha * alpha * pd;
    projector.project(y, tempx);
    Vec d(n), gy(n);
    bool moved = false;
    for (size_t i = 0; i < n; ++i) {
      d[i] = tempx[i] - y[i];
      gy[i] = g[i] - alpha * AP[i] + (e ? (*e)[i] : 0.0);
      moved = moved || d[i] != 0.0;
    }
    corr = 0.0;
    if (moved) {
      Vec Ad;
      mul(d, Ad);
      corr = dot(d, gy) + 0.5 * dot(d, Ad);
    }
    return dfy;
  }
  // CGMonotonicStep with the decrease test from scalars.  Same iterates and
  // control flow as the reference loop below; only "fy <= fx" is evaluated
  // as (f(P(y)) - f(x)) <= 0 without forming either function value.
  double CGMonotonicStepScalar(Vec &result, bool &result_is_prop) {
    Vec &AP = gp;
    Vec e;
    const Vec *ep = nullptr;
    if (!g_exact) {  // e = (A x - B) - g, constant along the CG run
      mul(result, e);
      for (size_t i = 0; i < e.size(); ++i) e[i] = (e[i] - B[i]) - g[i];
      ep = &e;
    }
    mul(p, AP);
    double pd = dot(p, AP);
    double alpha_cg = dot(z, g) / pd;
    double corr = 0.0, fx_off = 0.0;
    double dec = scalar_decrease(result, alpha_cg, pd, AP, ep, corr) + corr;
    result_is_prop = true;
    while (result_is_prop && residual_out > tolerance_factor && dec <= 0.0 &&
           iteration < (int)max_iterations) {
      result = y;
      fx_off = -corr;  // f(x) is now f(P(y)) while x is y
      for (size_t i = 0; i < g.size(); ++i) g[i] -= alpha_cg * AP[i];
      projector.PHI(g, phi);
      precond.solve(g, z, phi);
      const double b = dot(z, AP) / dot(p, AP);
      for (size_t i = 0; i < p.size(); ++i) p[i] = z[i] - b * p[i];
      residual_out = computeGradients(g, false);
      result_is_prop = proportional(result);
      mul(p, AP);
      pd = dot(p, AP);
      alpha_cg = dot(z, g) / pd;
      const double committed = dec;
      dec = scalar_decrease(result, alpha_cg, pd, AP, ep, corr) + corr + fx_off;
      ++num_cg;
      ++iteration;
      rec(1, committed);
    }
    rec(2, dec);
    return residual_out;
  }
  double CGMonotonicStep(Vec &result, bool &result_is_prop) {  // :272-316
    if (scalar_test) return CGMonotonicStepScalar(result, result_is_prop);
    Vec &AP = gp;
    mul(p, AP);
    double pd = dot(p, AP);
    double alpha_cg = dot(z, g) / pd;
    y.resize(result.size());
    for (size_t i = 0; i < y.size(); ++i) y[i] = result[i] - alpha_cg * p[i];
    double fy = projectFunValue(y);
    double fx = fval(result);
    result_is_prop = true;
    while (result_is_prop && residual_out > tolerance_factor && fy <= fx &&
           iteration < (int)max_iterations) {
      result = y;
      for (size_t i = 0; i < g.size(); ++i) g[i] -= alpha_cg * AP[i];
      projector.PHI(g, phi);
      precond.solve(g, z, phi);
      const double b = dot(z, AP) / dot(p, AP);
      for (size_t i = 0; i < p.size(); ++i) p[i] = z[i] - b * p[i];
      residual_out = computeGradients(g, false);
      result_is_prop = proportional(result);
      mul(p, AP);
      pd = dot(p, AP);
      alpha_cg = dot(z, g) / pd;
      for (size_t i = 0; i < y.size(); ++i) y[i] = result[i] - alpha_cg * p[i];
      const double dec = fy - fx;
      fx = fy;
      fy = projectFunValue(y);
      ++num_cg;
      ++iteration;
      rec(1, dec);
    }
    rec(2, fy - fx);
    return residual_out;
  }

  const MAT &A;
  const Vec &B;
  size_t max_iterations = 1000;
  double tolerance_factor = 1e-3;
  double gamma = 1.0, alpha_bar = 0.0, spec_rad = 0.0;
  PRECOND &precond;
  PROJ &projector;
  Vec g, p, z, beta, phi, gp, y, tempx;
  size_t iterations_out = 0;
  double residual_out = 0.0;
  int result_code = -1;
  int num_cg = 0, num_exp = 0, numprop = 0, iteration = 0;
  int power_iters = 0, spmv = 0;

  bool g_exact = true;  // g equals A x - B in exact arithmetic

 public:
  Trace *trace = nullptr;
  // Not the reference: evaluate CGMonotonicStep's test f(P(y)) <= f(x)
  // (MPRGPSolver.h:289, 305-309) from scalars, as the GPU solver does,
  // instead of comparing two separately rounded function values.  Off by
  // default; tests switch it on to show that the GPU takes the same steps.
  bool scalar_test = false;

 protected:
  void rec(int ev, double val) {
    if (trace) trace->push_back({(double)ev, (double)iteration, residual_out, val});
  }
};

// MPRGP::solve (MPRGPSolver.h:356-396), the non-monotone variant.
template <typename MAT, typename PROJ, typename PRECOND>
class MPRGP : public MPRGPBase<MAT, PROJ, PRECOND> {
  using MB = MPRGPBase<MAT, PROJ, PRECOND>;

 public:
  using MB::MB;
  int solve(Vec &result) {
    this->initialize(result);
    for (this->iteration = 0; this->iteration < (int)this->max_iterations; this->iteration++) {
      this->residual_out = this->computeGradients(this->g);
      if (this->residual_out <= this->tolerance_factor) {
        this->iterations_out = this->iteration;
        this->result_code = 0;
        break;
      }
      if (this->proportional(result)) {
        Vec &AP = this->gp;
        this->mul(this->p, AP);
        const double pd = dot(this->p, AP);
        const double alpha_cg = dot(this->z, this->g) / pd;
        const double alpha_f = this->projector.stepLimit(result, this->p, alpha_cg);
        if (alpha_cg <= alpha_f) this->CGStep(AP, alpha_cg, result);
        else this->ExpStep(AP, alpha_f, result);
      } else {
        this->PropStep(result);
      }
    }
    this->result_code = this->residual_out <= this->tolerance_factor ? 0 : -1;
    // The reference sets iterations_out only on convergence (:366).
    return this->result_code;
  }
};

// MPRGPMonotonic::solve (MPRGPSolver.h:412-454).
template <typename MAT, typename PROJ, typename PRECOND>
class MPRGPMonotonic : public MPRGPBase<MAT, PROJ, PRECOND> {
  using MB = MPRGPBase<MAT, PROJ, PRECOND>;

 public:
  using MB::MB;
  int solve(Vec &result) {
    this->initialize(result);
    bool y_valid = false;
    for (this->iteration = 0; this->iteration < (int)this->max_iterations;) {
      this->residual_out = this->computeGradients(this->g);
      if (this->residual_out <= this->tolerance_factor) break;
      bool result_is_prop = this->proportional(result);
      this->rec(5, result_is_prop ? 1.0 : 0.0);
      if (result_is_prop) {
        this->residual_out = this->CGMonotonicStep(result, result_is_prop);
        y_valid = true;
      }
      if (this->residual_out <= this->tolerance_factor) break;
      if (result_is_prop || !y_valid || !this->projector.isFeasible(this->y)) {
        this->ExpMonotonicStep(result);
        y_valid = true;  // ExpMonotonicStep writes y
        this->iteration++;
        this->rec(3, 0.0);
      } else {
        this->gradient(result);
        this->PropStep(result);
        this->iteration++;
        this->rec(4, 0.0);
      }
    }
    this->z = result;
    this->projector.project(this->z, result);
    this->result_code = this->residual_out <= this->tolerance_factor ? 0 : -1;
    this->iterations_out = this->iteration;
    return this->result_code;
  }
};

}  // namespace oracle
