// shim_eigen.hpp -- TEST INFRASTRUCTURE. A minimal stand-in for the handful of Eigen types
// that Sayram-2D's Solver.cc / Mesh.cc / Edge.h use, written for this project so that those
// reference sources compile here unmodified (Eigen itself is not available in this build
// environment). Only what those files call is provided:
//   Vector2d, RowVector2d, Matrix2d (comma initialiser), transpose products with (0) access,
//   VectorXd, Triplet, SparseMatrix<double, ColMajor> (setFromTriplets sums duplicates in
//   triplet order), SparseLU<...> (direct banded LU without pivoting; see banded_lu.h).
// Arithmetic follows the textbook definitions in left-to-right order: a row-vector/matrix
// product entry c is lhs(0)*M(0,c) + lhs(1)*M(1,c), a dot product is a0*b0 + a1*b1.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <initializer_list>
#include <stdexcept>
#include <vector>

#include "../banded_lu.h"

namespace Eigen {

enum StorageOptions { ColMajor = 0, RowMajor = 1 };

struct Scalar1x1 {  // result of a (1x2)*(2x1) product, read with (0)
  double v;
  double operator()(int) const { return v; }
};

struct RowVector2d;
struct Matrix2d;

struct Vector2d {
  double d[2];
  Vector2d() : d{0.0, 0.0} {}
  Vector2d(double a, double b) : d{a, b} {}
  double& operator()(int i) { return d[i]; }
  double operator()(int i) const { return d[i]; }
  double& operator[](int i) { return d[i]; }
  double operator[](int i) const { return d[i]; }
  Vector2d operator-(const Vector2d& o) const { return Vector2d(d[0] - o.d[0], d[1] - o.d[1]); }
  double squaredNorm() const { return d[0] * d[0] + d[1] * d[1]; }
  double norm() const { return std::sqrt(squaredNorm()); }
  RowVector2d transpose() const;
};

struct RowVector2d {
  double d[2];
  double operator()(int i) const { return d[i]; }
};

inline RowVector2d Vector2d::transpose() const { return RowVector2d{{d[0], d[1]}}; }

struct Matrix2d {
  double m[2][2] = {{0.0, 0.0}, {0.0, 0.0}};
  double operator()(int r, int c) const { return m[r][c]; }
  double& operator()(int r, int c) { return m[r][c]; }
  struct CommaInit {
    Matrix2d* M;
    int k;
    CommaInit& operator,(double v) {
      M->m[k / 2][k % 2] = v;
      ++k;
      return *this;
    }
  };
  CommaInit operator<<(double v) {
    m[0][0] = v;
    return CommaInit{this, 1};
  }
};

inline RowVector2d operator*(const RowVector2d& a, const Matrix2d& M) {
  return RowVector2d{{a.d[0] * M.m[0][0] + a.d[1] * M.m[1][0], a.d[0] * M.m[0][1] + a.d[1] * M.m[1][1]}};
}
inline Scalar1x1 operator*(const RowVector2d& a, const Vector2d& b) {
  return Scalar1x1{a.d[0] * b.d[0] + a.d[1] * b.d[1]};
}

struct VectorXd {
  std::vector<double> v;
  void resize(std::size_t n) { v.assign(n, 0.0); }
  void setZero() { std::fill(v.begin(), v.end(), 0.0); }
  std::size_t size() const { return v.size(); }
  double& operator()(std::size_t i) { return v[i]; }
  double operator()(std::size_t i) const { return v[i]; }
  double* data() { return v.data(); }
  const double* data() const { return v.data(); }
};

template <typename S>
struct Triplet {
  long r, c;
  S val;
  Triplet(long rr, long cc, S vv) : r(rr), c(cc), val(vv) {}
  long row() const { return r; }
  long col() const { return c; }
  S value() const { return val; }
};

template <typename S, int Opt = ColMajor>
struct SparseMatrix {
  long rows_ = 0, cols_ = 0;
  // compressed column storage
  std::vector<long> colptr, rowind;
  std::vector<double> vals;
  void resize(long r, long c) {
    rows_ = r;
    cols_ = c;
    colptr.assign(c + 1, 0);
    rowind.clear();
    vals.clear();
  }
  long rows() const { return rows_; }
  long cols() const { return cols_; }
  // Duplicates are summed sequentially in the order they appear in the triplet list.
  template <typename It>
  void setFromTriplets(It begin, It end) {
    std::vector<std::size_t> order;
    std::vector<Triplet<S>> t(begin, end);
    order.resize(t.size());
    for (std::size_t k = 0; k < t.size(); ++k) order[k] = k;
    std::stable_sort(order.begin(), order.end(), [&](std::size_t a, std::size_t b) {
      if (t[a].c != t[b].c) return t[a].c < t[b].c;
      return t[a].r < t[b].r;
    });
    colptr.assign(cols_ + 1, 0);
    rowind.clear();
    vals.clear();
    long lastr = -1, lastc = -1;
    for (std::size_t k : order) {
      const Triplet<S>& e = t[k];
      if (e.r == lastr && e.c == lastc) {
        vals.back() = vals.back() + e.val;
      } else {
        rowind.push_back(e.r);
        vals.push_back(e.val);
        colptr[e.c + 1]++;
        lastr = e.r;
        lastc = e.c;
      }
    }
    for (long c = 0; c < cols_; ++c) colptr[c + 1] += colptr[c];
  }
  void makeCompressed() {}
  double coeff(long r, long c) const {
    for (long k = colptr[c]; k < colptr[c + 1]; ++k)
      if (rowind[k] == r) return vals[k];
    return 0.0;
  }
};

template <typename I>
struct COLAMDOrdering {};

// Direct solve standing in for Eigen::SparseLU: banded LU without pivoting on the band of the
// assembled matrix (M is column diagonally dominant, see banded_lu.h).
template <typename Mat, typename Ord>
struct SparseLU {
  long n = 0, p = 0, q = 0;
  std::vector<double> band;
  int info_ = 0;
  void analyzePattern(const Mat&) {}
  void factorize(const Mat& M) {
    n = M.rows();
    p = q = 0;
    for (long c = 0; c < M.cols(); ++c)
      for (long k = M.colptr[c]; k < M.colptr[c + 1]; ++k) {
        const long r = M.rowind[k];
        if (r - c > p) p = r - c;
        if (c - r > q) q = c - r;
      }
    band.assign((std::size_t)n * (std::size_t)(p + q + 1), 0.0);
    for (long c = 0; c < M.cols(); ++c)
      for (long k = M.colptr[c]; k < M.colptr[c + 1]; ++k)
        band[blu_idx(M.rowind[k], c, p, q)] = M.vals[k];
    info_ = blu_factor(band.data(), n, p, q);
  }
  VectorXd solve(const VectorXd& b) const {
    VectorXd x;
    x.resize(b.size());
    blu_solve(band.data(), n, p, q, b.data(), x.data());
    return x;
  }
  int info() const { return info_; }
};

}  // namespace Eigen
