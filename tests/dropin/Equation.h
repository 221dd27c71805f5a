// TEST INFRASTRUCTURE: the Equation interface host/Solver.h calls (per-cell G, Dxx, Dxy, Dyy,
// inv_tau; bc_type, init_f, update(t), dirichlet_vertex_value), with the fields held in
// Xtensor2d members as the reference's Equation holds them.
#ifndef DROPIN_EQUATION_H
#define DROPIN_EQUATION_H

#include "BCTypes.h"
#include "Mesh.h"
#include "common.h"

class Equation {
 public:
  explicit Equation(const Mesh& m) {
    for (Xtensor2d* a : {&G_, &Dxx_, &Dxy_, &Dyy_, &inv_tau_}) a->resize({m.nx(), m.ny()});
  }
  virtual ~Equation() = default;
  double G(const Ind& k) const { return G_(k.i, k.j); }
  double Dxx(const Ind& k) const { return Dxx_(k.i, k.j); }
  double Dxy(const Ind& k) const { return Dxy_(k.i, k.j); }
  double Dyy(const Ind& k) const { return Dyy_(k.i, k.j); }
  double inv_tau(const Ind& k) const { return inv_tau_(k.i, k.j); }
  virtual BCType bc_type(BoundaryID side) const = 0;
  virtual double init_f(const Ind& ind) const = 0;
  virtual void update(double t) = 0;
  virtual bool dirichlet_vertex_value(BoundaryID side, std::size_t i, std::size_t j, double t,
                                      double* out_value) const = 0;

 protected:
  Xtensor2d G_, Dxx_, Dxy_, Dyy_, inv_tau_;
};

#endif
