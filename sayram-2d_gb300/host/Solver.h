/*
 * Solver.h -- drop-in for Sayram-2D's class Solver (source/Solver.h:18-26), backed by the GB300
 * C-ABI in sayram_gpu.h. Put this header in place of source/Solver.h, leave source/Solver.cc
 * out of the build and link libsayram_gpu.so; main.cc, Mesh and Equation stay unchanged.
 *
 *   Solver(const Mesh&, Equation*)   reads what the reference's Solver reads -- edges, dt
 *                                    (Mesh.h:38-63), G, Dxx, Dxy, Dyy, inv_tau, init_f, bc_type
 *                                    and the Dirichlet vertex values (Equation.h:44-65) -- and
 *                                    copies them to the device (Solver.cc:14-55)
 *   update()                         one backward-Euler step on the GPU (Solver.cc:270-290),
 *                                    then eq.update(t()) and the re-read of the Dirichlet
 *                                    vertex values (Solver.cc:286-289); with
 *                                    time_dependent_coeffs the coefficient fields too
 *   t(), f(), f(ind)                 as the reference; f() is a host mirror refreshed lazily
 *
 * Failures throw std::runtime_error with the library's message, as the reference throws on bad
 * grids (Grid2D.h:46-66) and missing Dirichlet values (Solver.cc:393). A step that ends above its
 * residual target is not an error here, matching the reference, which never checks
 * SparseLU::info() (Solver.cc:277); its status is in stats().
 */
#ifndef SOLVER_H
#define SOLVER_H

#include <stdexcept>
#include <string>
#include <vector>

#include "BCTypes.h"
#include "Equation.h"
#include "Mesh.h"
#include "common.h"
#include "sayram_gpu.h"

class Solver {
 public:
  Solver(const Mesh& m_in, Equation* eqp, int precision = SAYRAM_FP64, bool time_dependent_coeffs = false)
      : m(m_in), eq(*eqp), istep_(0), h_(nullptr), dirty_(true), tdep_(time_dependent_coeffs) {
    const std::size_t nx = m.nx(), ny = m.ny();
    f_.resize({nx, ny});
    std::vector<double> xe(nx + 1), ye(ny + 1);
    for (std::size_t i = 0; i <= nx; ++i) xe[i] = m.x_edge(i);
    for (std::size_t j = 0; j <= ny; ++j) ye[j] = m.y_edge(j);
    read_coeffs();
    std::vector<double> f0(nx * ny);
    for (std::size_t i = 0; i < nx; ++i)
      for (std::size_t j = 0; j < ny; ++j) f0[i * ny + j] = eq.init_f({i, j});
    read_dirichlet(0.0);
    sayram_problem p{};
    p.nx = (int)nx;
    p.ny = (int)ny;
    p.x_edges = xe.data();
    p.y_edges = ye.data();
    p.dt = m.dt();
    for (int s = 0; s < 4; ++s) {
      p.bc[s] = bc_[s];
      p.dirichlet[s] = bc_[s] == SAYRAM_DIRICHLET ? dir_[s].data() : nullptr;
    }
    p.G = G_.data();
    p.Dxx = Dxx_.data();
    p.Dxy = Dxy_.data();
    p.Dyy = Dyy_.data();
    p.inv_tau = itau_.data();
    p.f0 = f0.data();
    sayram_options o;
    sayram_default_options(&o);
    o.precision = precision;
    check(sayram_create(&p, &o, &h_), "sayram_create");
  }

  ~Solver() {
    if (h_) sayram_destroy(h_);
  }
  Solver(const Solver&) = delete;
  Solver& operator=(const Solver&) = delete;

  void update() {
    const int rc = sayram_update(h_);
    if (rc != SAYRAM_OK && rc != SAYRAM_ERR_NOT_CONVERGED) check(rc, "sayram_update");
    istep_ += 1;
    dirty_ = true;
    eq.update(t());
    if (tdep_) {
      read_coeffs();
      check(sayram_set_coeffs(h_, G_.data(), Dxx_.data(), Dxy_.data(), Dyy_.data(), itau_.data()), "sayram_set_coeffs");
    }
    read_dirichlet(t());
    for (int s = 0; s < 4; ++s)
      if (bc_[s] == SAYRAM_DIRICHLET)
        check(sayram_set_dirichlet(h_, s, dir_[s].data(), (int)dir_[s].size()), "sayram_set_dirichlet");
  }

  double t() const { return istep_ * m.dt(); }

  const Xtensor2d& f() const {
    if (dirty_) {
      check(sayram_get_f(h_, host_.data()), "sayram_get_f");
      const std::size_t nx = m.nx(), ny = m.ny();
      for (std::size_t i = 0; i < nx; ++i)
        for (std::size_t j = 0; j < ny; ++j) f_(i, j) = host_[i * ny + j];
      dirty_ = false;
    }
    return f_;
  }
  double f(const Ind& ind) const { return f()(ind.i, ind.j); }

  sayram_stats stats() const {
    sayram_stats s{};
    check(sayram_get_stats(h_, &s), "sayram_get_stats");
    return s;
  }

 private:
  const Mesh& m;
  Equation& eq;
  std::size_t istep_;
  sayram_solver h_;
  mutable bool dirty_;
  bool tdep_;
  mutable Xtensor2d f_;
  mutable std::vector<double> host_ = std::vector<double>(m.nx() * m.ny());
  std::vector<double> G_, Dxx_, Dxy_, Dyy_, itau_;
  int bc_[4] = {0, 0, 0, 0};
  std::vector<double> dir_[4];

  static void check(int rc, const char* what) {
    if (rc != SAYRAM_OK) throw std::runtime_error(std::string(what) + ": " + sayram_last_error());
  }

  void read_coeffs() {  // Equation fields, alpha-major (Solver::update_Lambda reads the same)
    const std::size_t nx = m.nx(), ny = m.ny(), n = nx * ny;
    G_.resize(n);
    Dxx_.resize(n);
    Dxy_.resize(n);
    Dyy_.resize(n);
    itau_.resize(n);
    for (std::size_t i = 0; i < nx; ++i)
      for (std::size_t j = 0; j < ny; ++j) {
        const std::size_t c = i * ny + j;
        G_[c] = eq.G({i, j});
        Dxx_[c] = eq.Dxx({i, j});
        Dxy_[c] = eq.Dxy({i, j});
        Dyy_[c] = eq.Dyy({i, j});
        itau_[c] = eq.inv_tau({i, j});
      }
  }

  void read_dirichlet(double tt) {  // fill_vertex_from_bcs, Solver.cc:385-422
    const std::size_t nx = m.nx(), ny = m.ny();
    const BoundaryID sides[4] = {BoundaryID::XMIN, BoundaryID::XMAX, BoundaryID::YMIN, BoundaryID::YMAX};
    for (int s = 0; s < 4; ++s) {
      bc_[s] = eq.bc_type(sides[s]) == BCType::Dirichlet ? SAYRAM_DIRICHLET : SAYRAM_ZEROFLUX;
      if (bc_[s] != SAYRAM_DIRICHLET) {
        dir_[s].clear();
        continue;
      }
      const std::size_t n = (s <= 1) ? ny + 1 : nx + 1;
      dir_[s].assign(n, 0.0);
      for (std::size_t k = 0; k < n; ++k) {
        const std::size_t i = (s == 0) ? 0 : (s == 1) ? nx : k;
        const std::size_t j = (s <= 1) ? k : (s == 2) ? 0 : ny;
        double u = 0.0;
        if (!eq.dirichlet_vertex_value(sides[s], i, j, tt, &u)) throw std::runtime_error("Dirichlet BC: missing value.");
        dir_[s][k] = u;
      }
    }
  }
};

#endif /* SOLVER_H */
