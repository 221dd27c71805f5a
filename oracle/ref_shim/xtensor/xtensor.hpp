// TEST INFRASTRUCTURE: a project-written stand-in for the xtensor containers that Sayram-2D's
// Solver/Mesh/Equation headers and its Albert_Young cases use (row-major 2-D storage,
// resize(shape), operator()(i,j), fill; a 1-D array with size(), [] and element-wise scaling).
#pragma once
#include <array>
#include <cstddef>
#include <initializer_list>
#include <vector>

namespace xt {

template <typename T, std::size_t Rank = 2>
struct xtensor {
  std::vector<T> data_;
  std::size_t n0 = 0, n1 = 0;
  void resize(const std::array<std::size_t, 2>& s) {
    n0 = s[0];
    n1 = s[1];
    data_.assign(n0 * n1, T());
  }
  void resize(std::initializer_list<std::size_t> s) {
    auto it = s.begin();
    std::array<std::size_t, 2> a = {*it, *(it + 1)};
    resize(a);
  }
  T& operator()(std::size_t i, std::size_t j) { return data_[i * n1 + j]; }
  const T& operator()(std::size_t i, std::size_t j) const { return data_[i * n1 + j]; }
  void fill(const T& v) {
    for (auto& x : data_) x = v;
  }
  T* data() { return data_.data(); }
  const T* data() const { return data_.data(); }
};

template <typename T>
struct xarray {
  std::vector<T> data_;
  std::size_t size() const { return data_.size(); }
  T& operator[](std::size_t i) { return data_[i]; }
  const T& operator[](std::size_t i) const { return data_[i]; }
};

// element-wise a * s and a / s, each element rounded once (as xtensor evaluates them)
inline xarray<double> operator*(const xarray<double>& a, double s) {
  xarray<double> r = a;
  for (auto& x : r.data_) x = x * s;
  return r;
}
inline xarray<double> operator/(const xarray<double>& a, double s) {
  xarray<double> r = a;
  for (auto& x : r.data_) x = x / s;
  return r;
}

}  // namespace xt
