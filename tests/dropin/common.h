// TEST INFRASTRUCTURE: a minimal stand-in for the types host/Solver.h takes from the reference's
// common.h (Ind, Xtensor2d), written for the drop-in test so that it compiles where the
// reference's headers (and their xtensor/Eigen dependencies) are absent. Only the members
// Solver.h uses exist: Ind{i, j}; Xtensor2d::resize({nx, ny}) and operator()(i, j), row-major.
#ifndef DROPIN_COMMON_H
#define DROPIN_COMMON_H

#include <array>
#include <cstddef>
#include <vector>

struct Ind {
  std::size_t i, j;
};

class Xtensor2d {
 public:
  void resize(const std::array<std::size_t, 2>& shape) {
    rows_ = shape[0];
    cols_ = shape[1];
    v_.assign(rows_ * cols_, 0.0);
  }
  double& operator()(std::size_t i, std::size_t j) { return v_[i * cols_ + j]; }
  double operator()(std::size_t i, std::size_t j) const { return v_[i * cols_ + j]; }
  std::size_t rows() const { return rows_; }
  std::size_t cols() const { return cols_; }

 private:
  std::size_t rows_ = 0, cols_ = 0;
  std::vector<double> v_;
};

#endif
