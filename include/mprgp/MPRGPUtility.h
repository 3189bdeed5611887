// include/mprgp/MPRGPUtility.h -- types and file formats of the C++ façade.
//
// The reference builds on Eigen (src/MPRGPSolver/MPRGPUtility.h); this façade
// keeps its names and semantics over light std::vector / CSR types so that it
// compiles without Eigen:
//   Vec<T>            ~ Eigen::Matrix<T,-1,1>
//   SparseMatrix<T>   ~ Eigen::SparseMatrix<T> (row-major CSR, built from triplets)
//   VVEC4X / VVVEC4X  ~ the reference's per-vertex plane lists (Vector4d n, p)
// and restates the QP file formats of writeQP/loadQP (MPRGPUtility.h:157-485:
// binary (A, B, J, c, x0), binary per-vertex planes, text with global
// planes) so QPs dumped by the reference's FEM driver
// (MprgpFemSolver.h:129-133) load here unchanged and files written here are
// byte for byte the reference's.
#pragma once

#include <algorithm>
#include <array>
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <string>
#include <tuple>
#include <vector>

namespace MATH {

template <typename T>
using Vec = std::vector<T>;

template <typename T>
struct Triplet {  // layout of Eigen::Triplet<T>: int row, int col, T value
  int r, c;
  T v;
  Triplet() = default;
  Triplet(int r_, int c_, T v_) : r(r_), c(c_), v(v_) {}
  int row() const { return r; }
  int col() const { return c; }
  T value() const { return v; }
};

// Compressed row storage; duplicates are summed as setFromTriplets does.
template <typename T>
class SparseMatrix {
 public:
  SparseMatrix() : ptr_(1, 0) {}
  SparseMatrix(int rows, int cols) : rows_(rows), cols_(cols), ptr_(rows + 1, 0) {}
  int rows() const { return rows_; }
  int cols() const { return cols_; }
  int nonZeros() const { return (int)idx_.size(); }
  void resize(int rows, int cols) {
    rows_ = rows;
    cols_ = cols;
    ptr_.assign(rows + 1, 0);
    idx_.clear();
    val_.clear();
  }
  template <typename It>
  void setFromTriplets(It begin, It end) {
    std::vector<std::tuple<int, int, T>> t;
    for (It it = begin; it != end; ++it) t.emplace_back(it->row(), it->col(), it->value());
    std::sort(t.begin(), t.end(), [](const std::tuple<int, int, T> &a,
                                     const std::tuple<int, int, T> &b) {
      return std::get<0>(a) != std::get<0>(b) ? std::get<0>(a) < std::get<0>(b)
                                              : std::get<1>(a) < std::get<1>(b);
    });
    ptr_.assign(rows_ + 1, 0);
    idx_.clear();
    val_.clear();
    for (size_t k = 0; k < t.size(); ++k) {
      const int r = std::get<0>(t[k]), c = std::get<1>(t[k]);
      if (!idx_.empty() && k > 0 && std::get<0>(t[k - 1]) == r && idx_.back() == c) {
        val_.back() += std::get<2>(t[k]);
        continue;
      }
      idx_.push_back(c);
      val_.push_back(std::get<2>(t[k]));
      ptr_[r + 1] = (int)idx_.size();
    }
    for (int r = 0; r < rows_; ++r) ptr_[r + 1] = std::max(ptr_[r + 1], ptr_[r]);
  }
  T coeff(int r, int c) const {
    for (int k = ptr_[r]; k < ptr_[r + 1]; ++k)
      if (idx_[k] == c) return val_[k];
    return T(0);
  }
  void multiply(const Vec<T> &x, Vec<T> &y) const {
    y.assign(rows_, T(0));
    for (int r = 0; r < rows_; ++r)
      for (int k = ptr_[r]; k < ptr_[r + 1]; ++k) y[r] += val_[k] * x[idx_[k]];
  }
  std::vector<Triplet<T>> triplets() const {
    std::vector<Triplet<T>> t;
    for (int r = 0; r < rows_; ++r)
      for (int k = ptr_[r]; k < ptr_[r + 1]; ++k) t.emplace_back(r, idx_[k], val_[k]);
    return t;
  }
  // The entries in the order the reference's files hold them: Eigen's
  // default column-major storage walked column by column, rows ascending.
  std::vector<Triplet<T>> triplets_by_column() const {
    std::vector<Triplet<T>> t = triplets();
    std::stable_sort(t.begin(), t.end(), [](const Triplet<T> &a, const Triplet<T> &b) {
      return a.c != b.c ? a.c < b.c : a.r < b.r;
    });
    return t;
  }
  const std::vector<int> &outerIndex() const { return ptr_; }
  const std::vector<int> &innerIndex() const { return idx_; }
  const std::vector<T> &values() const { return val_; }
  // Eigen's valuePtr(): the values in storage order, for in-place updates
  // that keep the sparsity (a Newton iteration's new A).
  T *valuePtr() { return val_.data(); }

 private:
  int rows_ = 0, cols_ = 0;
  std::vector<int> ptr_, idx_;
  std::vector<T> val_;
};

template <typename T>
using Vector4 = std::array<T, 4>;
template <typename T>
using VVEC4X = std::vector<Vector4<T>>;           // planes of one vertex (n, p)
template <typename T>
using VVVEC4X = std::vector<VVEC4X<T>>;           // per vertex

// COUNT_CONSTRAINTS (MPRGPUtility.h:98-106): the sum of the face codes.
inline int COUNT_CONSTRAINTS(const std::vector<char> &face) {
  int c = 0;
  for (char f : face) c += (int)f;
  return c;
}

// The same global planes for every one of num_nodes vertices
// (MPRGPUtility.h:110-117).
template <typename T>
VVVEC4X<T> &convert(const VVEC4X<T> &in, VVVEC4X<T> &out, const size_t num_nodes) {
  out.assign(num_nodes, in);
  return out;
}

// Planes -> (J, c) with J x >= c: row = n at the vertex's 3 columns, c = -p
// (MPRGPUtility.h:120-154).
template <typename T>
void convert(const VVVEC4X<T> &in, SparseMatrix<T> &J, Vec<T> &c) {
  std::vector<Triplet<T>> t;
  c.clear();
  for (size_t v = 0; v < in.size(); ++v)
    for (const auto &pl : in[v]) {
      const int row = (int)c.size();
      for (int d = 0; d < 3; ++d) t.emplace_back(row, (int)(3 * v + d), pl[d]);
      c.push_back(-pl[3]);
    }
  J.resize((int)c.size(), (int)(3 * in.size()));
  J.setFromTriplets(t.begin(), t.end());
}

// ---- binary QP files (MPRGPUtility.h:157-203, 258-485) -------------------
// Sparse matrix: size_t rows, cols, nnz, then nnz Triplet records.
template <typename T>
bool writeSparseMatrix(std::ofstream &out, const SparseMatrix<T> &A) {
  const size_t r = A.rows(), c = A.cols(), nz = A.nonZeros();
  out.write((const char *)&r, sizeof(r));
  out.write((const char *)&c, sizeof(c));
  out.write((const char *)&nz, sizeof(nz));
  const std::vector<Triplet<T>> t = A.triplets_by_column();
  if (!t.empty()) out.write((const char *)t.data(), sizeof(Triplet<T>) * nz);
  return out.good();
}
template <typename T>
bool loadSparseMatrix(std::ifstream &in, SparseMatrix<T> &A) {
  size_t r = 0, c = 0, nz = 0;
  in.read((char *)&r, sizeof(r));
  in.read((char *)&c, sizeof(c));
  in.read((char *)&nz, sizeof(nz));
  if (!in.good()) return false;
  A.resize((int)r, (int)c);
  if (nz > 0) {
    std::vector<Triplet<T>> t(nz);
    in.read((char *)t.data(), sizeof(Triplet<T>) * nz);
    A.setFromTriplets(t.begin(), t.end());
  }
  return in.good();
}
template <typename T>
void writeVec(std::ofstream &out, const Vec<T> &v) {
  if (!v.empty()) out.write((const char *)v.data(), sizeof(T) * v.size());
}
template <typename T>
void readVec(std::ifstream &in, Vec<T> &v, size_t n) {
  v.resize(n);
  if (n) in.read((char *)v.data(), sizeof(T) * n);
}

// (A, B, J, c, x0) form (MPRGPUtility.h:407-485).
template <typename T>
bool writeQP(const SparseMatrix<T> &A, const Vec<T> &B, const SparseMatrix<T> &J,
             const Vec<T> &c, const Vec<T> &x0, const std::string &file_name) {
  std::ofstream out(file_name.c_str(), std::ios::out | std::ios::binary);
  if (!out.is_open()) return false;
  writeSparseMatrix(out, A);
  writeVec(out, B);
  writeSparseMatrix(out, J);
  writeVec(out, c);
  writeVec(out, x0);
  return out.good();
}
template <typename T>
bool loadQP(SparseMatrix<T> &A, Vec<T> &B, SparseMatrix<T> &J, Vec<T> &c, Vec<T> &x0,
            const std::string &file_name) {
  std::ifstream in(file_name.c_str(), std::ios::in | std::ios::binary);
  if (!in.is_open()) return false;
  if (!loadSparseMatrix(in, A)) return false;
  readVec(in, B, A.rows());
  if (!loadSparseMatrix(in, J)) return false;
  readVec(in, c, J.rows());
  readVec(in, x0, A.rows());
  return in.good();
}

// Per-vertex plane form (MPRGPUtility.h:258-402): A, B, then for each vertex
// size_t count and count (n, p) records, then x0.
template <typename T>
bool writeQP(const SparseMatrix<T> &A, const Vec<T> &B, const VVVEC4X<T> &planes,
             const Vec<T> &x0, const std::string &file_name) {
  std::ofstream out(file_name.c_str(), std::ios::out | std::ios::binary);
  if (!out.is_open()) return false;
  writeSparseMatrix(out, A);
  writeVec(out, B);
  for (const auto &pv : planes) {
    const size_t p = pv.size();
    out.write((const char *)&p, sizeof(p));
    for (const auto &pl : pv) out.write((const char *)pl.data(), sizeof(T) * 4);
  }
  writeVec(out, x0);
  return out.good();
}
template <typename T>
bool loadQP(SparseMatrix<T> &A, Vec<T> &B, VVVEC4X<T> &planes, Vec<T> &x0,
            const std::string &file_name) {
  std::ifstream in(file_name.c_str(), std::ios::in | std::ios::binary);
  if (!in.is_open()) return false;
  if (!loadSparseMatrix(in, A)) return false;
  readVec(in, B, A.rows());
  if (A.rows() % 3 != 0) return false;
  planes.assign(A.rows() / 3, VVEC4X<T>());
  for (auto &pv : planes) {
    size_t p = 0;
    in.read((char *)&p, sizeof(p));
    if (!in.good() || p > 1024) return false;
    pv.resize(p);
    for (auto &pl : pv) in.read((char *)pl.data(), sizeof(T) * 4);
  }
  readVec(in, x0, A.rows());
  return in.good();
}

// ---- text QP file with global planes (MPRGPUtility.h:208-257, 295-357) ----
// "dimension n", "planes m", "A", "non_zeros nnz", one "row\tcol\tvalue" line
// per entry (column by column), "B" and one tab-separated line of n values,
// "P" and one "nx\tny\tnz\tp" line per plane, "x0" and one line of n values;
// numbers with 12 significant digits.  The planes apply to every vertex
// (convert(planes, per_node, n / 3)).
template <typename T>
bool writeQP(const SparseMatrix<T> &A, const Vec<T> &B, const VVEC4X<T> &planes,
             const Vec<T> &x0, const std::string &file_name) {
  std::ofstream out(file_name.c_str());
  if (!out.is_open()) return false;
  out << "dimension " << A.rows() << "\n";
  out << "planes " << planes.size() << "\n";
  out << "A\n";
  out << "non_zeros " << A.nonZeros() << "\n";
  out.precision(12);
  for (const Triplet<T> &t : A.triplets_by_column())
    out << t.row() << "\t" << t.col() << "\t" << t.value() << "\n";
  auto line = [&out](const Vec<T> &v) {
    for (size_t i = 0; i < v.size(); ++i) out << (i ? "\t" : "") << v[i];
    out << "\n";
  };
  out << "B\n";
  line(B);
  out << "P\n";
  for (const auto &pl : planes)
    out << pl[0] << "\t" << pl[1] << "\t" << pl[2] << "\t" << pl[3] << "\n";
  out << "x0\n";
  line(x0);
  return out.good();
}
template <typename T>
bool loadQP(SparseMatrix<T> &A, Vec<T> &B, VVEC4X<T> &planes, Vec<T> &x0,
            const std::string &file_name) {
  std::ifstream in(file_name.c_str());
  if (!in.is_open()) return false;
  std::string tag;
  long long n = -1, m = -1, nnz = -1;
  in >> tag >> n >> tag >> m;
  in >> tag >> tag >> nnz;
  if (!in.good() || n < 0 || m < 0 || nnz < 0) return false;
  std::vector<Triplet<T>> t;
  t.reserve((size_t)nnz);
  for (long long k = 0; k < nnz; ++k) {
    long long r, c;
    T v;
    in >> r >> c >> v;
    if (!in.good() || r < 0 || c < 0 || r >= n || c >= n) return false;
    t.emplace_back((int)r, (int)c, v);
  }
  A.resize((int)n, (int)n);
  A.setFromTriplets(t.begin(), t.end());
  in >> tag;
  B.resize((size_t)n);
  for (auto &v : B) in >> v;
  in >> tag;
  planes.resize((size_t)m);
  for (auto &pl : planes) in >> pl[0] >> pl[1] >> pl[2] >> pl[3];
  in >> tag;
  x0.resize((size_t)n);
  for (auto &v : x0) in >> v;
  return !in.fail();
}

}  // namespace MATH
