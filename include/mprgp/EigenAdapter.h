// include/mprgp/EigenAdapter.h -- optional conversions between Eigen types and
// the façade's, for drivers that keep their system in Eigen as the
// reference's FEM driver does (Eigen::SparseMatrix<double> LHS_mat and
// Eigen::VectorXd RHS / new_pos, MprgpFemSolver.cpp:521-533; per-vertex
// planes as std::vector<std::vector<Eigen::Vector4d>>, MprgpFemSolver.h:107).
//
// Include it after the Eigen headers; the rest of the façade needs no Eigen.
//
//   #include <Eigen/Sparse>
//   #include "mprgp/EigenAdapter.h"
//   MATH::SparseMatrix<double> A = MATH::from_eigen(LHS_mat);
//   MATH::Vec<double> b = MATH::from_eigen(RHS), x = MATH::from_eigen(new_pos);
//   ... solve ...
//   MATH::to_eigen(x, new_pos);
#pragma once

#include <algorithm>
#include <vector>

#include "MPRGPUtility.h"

namespace MATH {

// Eigen::SparseMatrix (either storage order) -> CSR, entry for entry.
template <typename T, int Options, typename StorageIndex>
SparseMatrix<T> from_eigen(const Eigen::SparseMatrix<T, Options, StorageIndex> &A) {
  using EM = Eigen::SparseMatrix<T, Options, StorageIndex>;
  std::vector<Triplet<T>> t;
  t.reserve((size_t)A.nonZeros());
  for (int k = 0; k < (int)A.outerSize(); ++k)
    for (typename EM::InnerIterator it(A, k); it; ++it)
      t.emplace_back((int)it.row(), (int)it.col(), it.value());
  SparseMatrix<T> out((int)A.rows(), (int)A.cols());
  out.setFromTriplets(t.begin(), t.end());
  return out;
}

// Eigen dense vector -> Vec.
template <typename Derived>
Vec<typename Derived::Scalar> from_eigen(const Eigen::MatrixBase<Derived> &v) {
  Vec<typename Derived::Scalar> out((size_t)v.size());
  for (int i = 0; i < (int)v.size(); ++i) out[(size_t)i] = v(i);
  return out;
}

// Vec -> an Eigen dense vector (resized to fit).
template <typename T, typename EigenVector>
void to_eigen(const Vec<T> &v, EigenVector &out) {
  out.resize((int)v.size());
  for (size_t i = 0; i < v.size(); ++i) out((int)i) = v[i];
}

// Per-vertex planes (n, p) as Eigen 4-vectors -> the façade's VVVEC4X.
template <typename T, typename V4, typename A1, typename A2>
VVVEC4X<T> planes_from_eigen(const std::vector<std::vector<V4, A1>, A2> &in) {
  VVVEC4X<T> out(in.size());
  for (size_t v = 0; v < in.size(); ++v)
    for (const V4 &q : in[v]) out[v].push_back(Vector4<T>{q(0), q(1), q(2), q(3)});
  return out;
}

}  // namespace MATH
