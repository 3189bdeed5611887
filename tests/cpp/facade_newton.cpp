// Times the C++ façade the way the reference's FEM driver calls it
// (MprgpFemSolver.cpp:521-533): one QP file (the reference's binary
// (A, B, J, c, x0) layout), then `steps` solves of MPRGPGeneralCon<double>
// with the same sparsity and new values each time, as a Newton loop updates
// A in place.  Each solve's wall time covers the whole façade call: the
// host-side 3x3-block and plane conversion, the copies to and from the GPU
// and the solve.  Prints one line: key=value pairs.
// Usage: facade_newton <qp file> <steps> <relative tol>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "mprgp/MPRGPSolver.h"

using namespace MATH;

int main(int argc, char **argv) {
  if (argc < 4) return 2;
  const std::string file = argv[1];
  const int steps = std::atoi(argv[2]);
  const double rel_tol = std::atof(argv[3]);
  SparseMatrix<double> A, J;
  Vec<double> B, c, x0;
  if (!loadQP(A, B, J, c, x0, file)) {
    std::printf("error=load\n");
    return 1;
  }
  double nb = 0.0;
  for (double v : B) nb += v * v;
  const double tol = rel_tol * std::sqrt(nb);
  std::vector<double> base(A.values());
  std::vector<double> ms;
  int bad = 0;
  long long iters = 0;
  for (int s = 0; s < steps; ++s) {
    // the next Newton iteration's matrix: same pattern, new values (SPD)
    const double f = 1.0 + 1e-3 * s;
    double *v = A.valuePtr();
    for (size_t k = 0; k < base.size(); ++k) v[k] = base[k] * f;
    Vec<double> x = x0;
    const auto t0 = std::chrono::steady_clock::now();
    const int rc = MPRGPGeneralCon<double>::solve<SparseMatrix<double>, true>(A, B, J, c, x, tol,
                                                                           20000);
    const auto t1 = std::chrono::steady_clock::now();
    ms.push_back(std::chrono::duration<double, std::milli>(t1 - t0).count());
    bad += rc != 0;
    iters += gpu::last_stats().iterations;
  }
  double later = 0.0;
  for (int s = 1; s < steps; ++s) later += ms[s];
  later /= std::max(1, steps - 1);
  const gpu::BlockPattern &P = gpu::block_pattern();
  std::printf("solves=%d failed=%d first_ms=%.3f later_ms=%.3f iterations=%lld pattern_builds=%lld "
              "pattern_refills=%lld n=%d nnz=%d constraints=%d\n",
              steps, bad, ms.empty() ? 0.0 : ms[0], later, iters, P.builds, P.refills, A.rows(),
              A.nonZeros(), J.rows());
  return bad ? 1 : 0;
}
