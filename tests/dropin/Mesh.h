// TEST INFRASTRUCTURE: the part of the reference's Mesh interface host/Solver.h reads -- nx(),
// ny(), x_edge(i), y_edge(j), dt() -- over explicit edge arrays.
#ifndef DROPIN_MESH_H
#define DROPIN_MESH_H

#include <cstddef>
#include <utility>
#include <vector>

class Mesh {
 public:
  Mesh(std::vector<double> x_edges, std::vector<double> y_edges, double dt)
      : xe_(std::move(x_edges)), ye_(std::move(y_edges)), dt_(dt) {}
  std::size_t nx() const { return xe_.size() - 1; }
  std::size_t ny() const { return ye_.size() - 1; }
  double x_edge(std::size_t i) const { return xe_[i]; }
  double y_edge(std::size_t j) const { return ye_[j]; }
  double dt() const { return dt_; }

 private:
  std::vector<double> xe_, ye_;
  double dt_;
};

#endif
