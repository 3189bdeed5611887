// Drop-in test of the C++ façade: the reference's own unit tests
// (test_case/MPRGPTest.cpp) written against include/mprgp/MPRGPSolver.h,
// plus the reference's binary QP file round trip (MPRGPUtility.h:407-485)
// and the file-form solve (MPRGPSolver.h:576-589).  Given the fixture
// directory tests/golden/qp_files as argv[1], it also solves the fixtures the
// way a reference user would -- the decoupled file form on the (J, c) file,
// and the text file's global planes through convert() and MPRGPGeneralCon --
// and writes each solution to x_<form>.txt for the oracle comparison.
// Prints one line per check; exits non-zero on failure.
#include <cmath>
#include <cstdio>
#include <random>

#include "mprgp/ICASolver.h"
#include "mprgp/MPRGPSolver.h"

using namespace MATH;

static int failures = 0;
#define CHECK(cond)                                                  \
  do {                                                               \
    if (!(cond)) {                                                   \
      std::printf("FAIL %s:%d %s\n", __FILE__, __LINE__, #cond);     \
      ++failures;                                                    \
    }                                                                \
  } while (0)

static SparseMatrix<double> from_dense(const std::vector<double> &M, int r, int c) {
  std::vector<Triplet<double>> t;
  for (int i = 0; i < r; ++i)
    for (int j = 0; j < c; ++j)
      if (M[i * c + j] != 0.0) t.emplace_back(i, j, M[i * c + j]);
  SparseMatrix<double> S(r, c);
  S.setFromTriplets(t.begin(), t.end());
  return S;
}

static void save(const Vec<double> &x, const char *path) {
  FILE *f = std::fopen(path, "w");
  for (double v : x) std::fprintf(f, "%.17g\n", v);
  std::fclose(f);
}

static double norm(const Vec<double> &v) {
  double s = 0.0;
  for (double t : v) s += t * t;
  return std::sqrt(s);
}

int main(int argc, char **argv) {
  std::mt19937 gen(7);
  std::uniform_real_distribution<double> U(-1.0, 1.0);
  // test_solver (MPRGPTest.cpp:70-98): random SPD 5x5, J = I.
  const int n = 5;
  std::vector<double> Md(n * n), MtM(n * n, 0.0), I(n * n, 0.0);
  for (int i = 0; i < n * n; ++i) Md[i] = U(gen) + ((i % (n + 1)) == 0 ? 3.0 : 0.0);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j)
      for (int k = 0; k < n; ++k) MtM[i * n + j] += Md[k * n + i] * Md[k * n + j];
  for (int i = 0; i < n; ++i) I[i * n + i] = 1.0;
  const SparseMatrix<double> A = from_dense(MtM, n, n), J = from_dense(I, n, n);
  Vec<double> B(n), c(n), x(n);
  for (int i = 0; i < n; ++i) { B[i] = U(gen); c[i] = U(gen); x[i] = U(gen); }
  typedef FixedSparseMatrix<double> MAT;
  MAT FA(A);
  {
    Vec<double> y = x;
    const int rc = MPRGPGeneralCon<double>::solve<MAT, true>(FA, B, J, c, y, 1e-10, 1000);
    std::printf("general: code %d\n", rc);
    CHECK(rc == 0);
    for (int i = 0; i < n; ++i) CHECK(y[i] >= c[i] - 1e-9);
  }
  {
    Vec<double> y = x;
    const int rc = MPRGPDecoupledCon<double>::solve<MAT, true>(FA, B, J, c, y, 1e-10, 1000);
    std::printf("decoupled: code %d\n", rc);
    CHECK(rc == 0);
    for (int i = 0; i < n; ++i) CHECK(y[i] >= c[i] - 1e-9);
  }
  {  // lower bound and box façades on the same system
    Vec<double> y = x, L = c, H(n, 0.7);
    for (int i = 0; i < n; ++i) y[i] = std::max(y[i], L[i]);
    CHECK(MPRGPLowerBound<double>::solve(FA, B, L, y, 1e-10, 1000) == 0);
    Vec<double> z(n);
    for (int i = 0; i < n; ++i) z[i] = std::min(std::max(x[i], L[i]), std::max(L[i], H[i]));
    for (int i = 0; i < n; ++i) H[i] = std::max(L[i], H[i]);
    CHECK(MPRGPBoxBound<double>::solve(FA, B, L, H, z, 1e-10, 1000) == 0);
    for (int i = 0; i < n; ++i) CHECK(z[i] >= L[i] - 1e-9 && z[i] <= H[i] + 1e-9);
  }
  {  // generic classes with projector objects
    Vec<double> JJt(n, 1.0), y = x;
    DecoupledConProjector<double> proj(J, JJt, c);
    proj.project(x, y);
    DiagonalDecouplePreconSolver<double, MAT> pre(FA, proj.getFace(), J);
    MPRGPMonotonic<double, MAT, DecoupledConProjector<double>,
                   DiagonalDecouplePreconSolver<double, MAT>>
        solver(FA, B, pre, proj, 1000, 1e-10);
    CHECK(solver.solve(y) == 0);
    CHECK(solver.residualOut() <= 1e-10);
    std::printf("monotone decoupled: iterations %zu active %d\n", solver.iterationsOut(),
                COUNT_CONSTRAINTS(proj.getFace()));
  }
  {  // QP file round trip and the file-form solve (MPRGPSolver.h:576-589)
    const std::string path = "facade_qp.b";
    CHECK(writeQP(A, B, J, c, x, path));
    SparseMatrix<double> A2, J2;
    Vec<double> B2, c2, x2;
    CHECK(loadQP(A2, B2, J2, c2, x2, path));
    CHECK(A2.nonZeros() == A.nonZeros() && J2.rows() == J.rows() && x2 == x && c2 == c);
    Vec<double> y;
    const int rc = MPRGPDecoupledCon<double>::solve<true>(path, y, 1e-10, 1000);
    std::printf("file-form solve: code %d\n", rc);
    CHECK(rc == 0 && (int)y.size() == n);
    std::remove(path.c_str());
  }
  {  // MPRGP vs ICA on one QP (test_case/MPRGP_ICA_Compare.cpp:12-83), n = 3 * 3
    const int m3 = 9;
    std::vector<double> Gd(m3 * m3), G(m3 * m3, 0.0), Jd(3 * m3, 0.0);
    for (int i = 0; i < m3 * m3; ++i) Gd[i] = U(gen) + ((i % (m3 + 1)) == 0 ? 3.0 : 0.0);
    for (int i = 0; i < m3; ++i)
      for (int j = 0; j < m3; ++j)
        for (int k = 0; k < m3; ++k) G[i * m3 + j] += Gd[k * m3 + i] * Gd[k * m3 + j];
    for (int v = 0; v < 3; ++v) Jd[v * m3 + 3 * v + 1] = 1.0;  // y_v >= p_v
    const SparseMatrix<double> A3 = from_dense(G, m3, m3), J3 = from_dense(Jd, 3, m3);
    Vec<double> B3(m3), p3(3), x0(m3, 0.0);
    for (int i = 0; i < m3; ++i) B3[i] = U(gen);
    for (int v = 0; v < 3; ++v) p3[v] = 0.5 * U(gen);
    Vec<double> xm = x0;
    const int rc = MPRGPDecoupledCon<double>::solve<SparseMatrix<double>, true>(A3, B3, J3, p3, xm, 1e-12, 10000);
    CHECK(rc == 0);
    ICASolver ica(100000, 1e-12, 20, 1e-14);
    ica.setName("ica with con");
    ica.reset(A3, B3);
    Vec<double> xi = x0;
    CHECK(ica.solve(J3, p3, xi));
    double d = 0.0, nx = 0.0, compl_ = 0.0;
    for (int i = 0; i < m3; ++i) {
      d += (xi[i] - xm[i]) * (xi[i] - xm[i]);
      nx += xm[i] * xm[i];
    }
    for (int v = 0; v < 3; ++v) {
      CHECK(ica.getLambda()[v] >= 0.0);
      CHECK(xi[3 * v + 1] >= p3[v] - 1e-9);
      compl_ += ica.getLambda()[v] * (xi[3 * v + 1] - p3[v]);
    }
    CHECK(std::sqrt(d) <= 1e-8 * std::sqrt(nx));
    CHECK(std::fabs(compl_) <= 1e-9);
    CHECK(ica.getResidual() <= 1e-12);
    std::printf("ica: iterations %d residual %.3e |x_ica - x_mprgp| %.3e\n", ica.getIterations(),
                ica.getResidual(), std::sqrt(d));
  }
  if (argc > 1) {  // the reference file forms, solved as a reference user would
    const std::string dir = argv[1];
    {
      SparseMatrix<double> A, J;
      Vec<double> B, c, x0;
      CHECK(loadQP(A, B, J, c, x0, dir + "/beam_1x2x2.jc.b"));
      Vec<double> y;
      const int rc = MPRGPDecoupledCon<double>::solve<true>(dir + "/beam_1x2x2.jc.b", y,
                                                            1e-10 * norm(B), 10000);
      std::printf("file-form (J, c) solve: code %d\n", rc);
      CHECK(rc == 0 && y.size() == B.size());
      save(y, "x_jc.txt");
    }
    {
      SparseMatrix<double> A, J;
      Vec<double> B, c, x;
      VVEC4X<double> planes;
      VVVEC4X<double> per_node;
      CHECK(loadQP(A, B, planes, x, dir + "/beam_1x2x2.txt"));
      convert(planes, per_node, (size_t)A.rows() / 3);
      convert(per_node, J, c);
      FixedSparseMatrix<double> FA(A);
      const int rc = MPRGPGeneralCon<double>::solve<FixedSparseMatrix<double>, true>(
          FA, B, J, c, x, 1e-10 * norm(B), 10000);
      std::printf("text-form solve (global planes): code %d\n", rc);
      CHECK(rc == 0);
      save(x, "x_text.txt");
    }
  }
  std::printf("%s (%d failures)\n", failures ? "FAILED" : "OK", failures);
  return failures ? 1 : 0;
}
