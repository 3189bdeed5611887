// The reference's three QP file forms through the façade's loaders and
// writers (include/mprgp/MPRGPUtility.h), host code only: each fixture of
// tests/golden/qp_files loads, and writing what was loaded gives the same
// bytes back.  Usage: test_qp_files <fixture dir> <scratch dir>.
#include <cstdio>
#include <fstream>
#include <iterator>
#include <string>

#include "mprgp/MPRGPUtility.h"

using namespace MATH;

static int failures = 0;
#define CHECK(cond)                                              \
  do {                                                           \
    if (!(cond)) {                                               \
      std::printf("FAIL %s:%d %s\n", __FILE__, __LINE__, #cond); \
      ++failures;                                                \
    }                                                            \
  } while (0)

static std::string bytes(const std::string &path) {
  std::ifstream in(path.c_str(), std::ios::binary);
  return std::string(std::istreambuf_iterator<char>(in), std::istreambuf_iterator<char>());
}

int main(int argc, char **argv) {
  if (argc < 3) return 2;
  const std::string dir = argv[1], tmp = argv[2];
  {  // binary (A, B, J, c, x0), MPRGPUtility.h:407-485
    SparseMatrix<double> A, J;
    Vec<double> B, c, x0;
    const std::string f = dir + "/beam_1x2x2.jc.b", g = tmp + "/jc.b";
    CHECK(loadQP(A, B, J, c, x0, f));
    CHECK(A.rows() == 54 && A.cols() == 54 && J.rows() == 18 && J.cols() == 54);
    CHECK(B.size() == 54 && c.size() == 18 && x0.size() == 54);
    CHECK(writeQP(A, B, J, c, x0, g));
    CHECK(bytes(f) == bytes(g));
    std::printf("jc: n %d nnz %d constraints %d B[0] %.17g\n", A.rows(), A.nonZeros(), J.rows(),
                B[0]);
  }
  {  // binary per-vertex planes, MPRGPUtility.h:258-292, 359-402
    SparseMatrix<double> A;
    Vec<double> B, x0;
    VVVEC4X<double> planes;
    const std::string f = dir + "/beam_1x2x2.planes.b", g = tmp + "/planes.b";
    CHECK(loadQP(A, B, planes, x0, f));
    CHECK(planes.size() == 18);
    size_t m = 0;
    for (const auto &pv : planes) m += pv.size();
    CHECK(writeQP(A, B, planes, x0, g));
    CHECK(bytes(f) == bytes(g));
    SparseMatrix<double> J;
    Vec<double> c;
    convert(planes, J, c);
    CHECK((size_t)J.rows() == m && c.size() == m);
    std::printf("planes: vertices %zu planes %zu\n", planes.size(), m);
  }
  {  // text with global planes, MPRGPUtility.h:208-257, 295-357
    SparseMatrix<double> A;
    Vec<double> B, x0;
    VVEC4X<double> planes;
    const std::string f = dir + "/beam_1x2x2.txt", g = tmp + "/qp.txt";
    CHECK(loadQP(A, B, planes, x0, f));
    CHECK(A.rows() == 54 && planes.size() == 2 && B.size() == 54 && x0.size() == 54);
    CHECK(writeQP(A, B, planes, x0, g));
    CHECK(bytes(f) == bytes(g));
    VVVEC4X<double> per_node;
    convert(planes, per_node, (size_t)A.rows() / 3);
    SparseMatrix<double> J;
    Vec<double> c;
    convert(per_node, J, c);
    CHECK(J.rows() == 36 && c.size() == 36 && c[1] == 0.01);
    std::printf("text: n %d nnz %d global planes %zu\n", A.rows(), A.nonZeros(), planes.size());
  }
  {  // a missing file is a false return, as in the reference
    SparseMatrix<double> A, J;
    Vec<double> B, c, x0;
    CHECK(!loadQP(A, B, J, c, x0, tmp + "/missing.b"));
  }
  std::printf("%s (%d failures)\n", failures ? "FAILED" : "OK", failures);
  return failures ? 1 : 0;
}
