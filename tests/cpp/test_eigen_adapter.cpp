// include/mprgp/EigenAdapter.h over a stand-in for the Eigen names it uses
// (tests/cpp/fake_eigen): a column-major and a row-major sparse matrix
// convert entry for entry, vectors round-trip, per-vertex Vector4d planes
// become the façade's VVVEC4X.  Host code only.
#include <Eigen/Sparse>

#include <cstdio>
#include <vector>

#include "mprgp/EigenAdapter.h"

static int failures = 0;
#define CHECK(cond)                                              \
  do {                                                           \
    if (!(cond)) {                                               \
      std::printf("FAIL %s:%d %s\n", __FILE__, __LINE__, #cond); \
      ++failures;                                                \
    }                                                            \
  } while (0)

template <int Options>
static void check_matrix() {
  const int n = 12;
  Eigen::SparseMatrix<double, Options> E(n, n);
  std::vector<std::vector<double>> dense(n, std::vector<double>(n, 0.0));
  for (int r = 0; r < n; ++r)
    for (int c = 0; c < n; ++c)
      if ((r * 7 + c * 3) % 5 == 0 || r == c) {
        const double v = 1.0 + r - 0.25 * c;
        E.insert(r, c) = v;
        dense[r][c] = v;
      }
  const MATH::SparseMatrix<double> A = MATH::from_eigen(E);
  CHECK(A.rows() == n && A.cols() == n);
  CHECK(A.nonZeros() == (int)E.nonZeros());
  // every entry, through the façade's column-ordered triplets
  int seen = 0;
  for (const auto &t : A.triplets_by_column()) {
    CHECK(t.value() == dense[t.row()][t.col()]);
    ++seen;
  }
  CHECK(seen == A.nonZeros());
}

int main() {
  check_matrix<Eigen::ColMajor>();
  check_matrix<Eigen::RowMajor>();
  Eigen::VectorXd v(5);
  for (int i = 0; i < 5; ++i) v(i) = 0.5 * i - 1.0;
  const MATH::Vec<double> f = MATH::from_eigen(v);
  CHECK(f.size() == 5 && f[0] == -1.0 && f[4] == 1.0);
  Eigen::VectorXd back;
  MATH::to_eigen(f, back);
  CHECK(back.size() == 5);
  for (int i = 0; i < 5; ++i) CHECK(back(i) == v(i));
  std::vector<std::vector<Eigen::Vector4d>> planes(3);
  planes[0].push_back(Eigen::Vector4d(0, 1, 0, 0.5));
  planes[2].push_back(Eigen::Vector4d(1, 0, 0, -2.0));
  planes[2].push_back(Eigen::Vector4d(0, 0, 1, 0.25));
  const MATH::VVVEC4X<double> p = MATH::planes_from_eigen<double>(planes);
  CHECK(p.size() == 3 && p[0].size() == 1 && p[1].empty() && p[2].size() == 2);
  CHECK(p[0][0][1] == 1.0 && p[0][0][3] == 0.5 && p[2][1][2] == 1.0 && p[2][1][3] == 0.25);
  if (failures) return 1;
  std::printf("ok\n");
  return 0;
}
