// ref_harness.cc -- TEST INFRASTRUCTURE. Drives the reference's own Solver (Sayram-2D
// source/Solver.cc, source/Mesh.cc, compiled unmodified against the shim headers in ref_shim/)
// on arrays supplied by the tests, so that fixtures come from the reference's code itself.
//
// Built only where the reference sources are present (Makefile target `ref`), into oracle/_ref/.
// The Equation subclass below plays the role of a case (like source/Cases/Albert_Young.cc):
// it serves G, D, 1/tau, f0, BC types and Dirichlet vertex values from caller arrays.
#include <cstring>
#include <exception>
#include <string>
#include <vector>

#include "common.h"
#include "Grid2D.h"
#include "BCTypes.h"
// Solver keeps M_ and R_ private; the fixtures need them, so open the class for this harness.
#define private public
#include "Solver.h"
#undef private

namespace {

class ArrayEquation : public Equation {
 public:
  ArrayEquation(const Mesh& m, const double* G, const double* Dxx, const double* Dxy,
                const double* Dyy, const double* inv_tau, const double* f0, const int* bc,
                const double* const* dir)
      : Equation(m), m_(m), f0_(f0) {
    const std::size_t nx = m.nx(), ny = m.ny();
    for (std::size_t i = 0; i < nx; ++i)
      for (std::size_t j = 0; j < ny; ++j) {
        const std::size_t c = i * ny + j;
        G_(i, j) = G[c];
        Dxx_(i, j) = Dxx[c];
        Dxy_(i, j) = Dxy[c];
        Dyy_(i, j) = Dyy[c];
        inv_tau_(i, j) = inv_tau[c];
      }
    for (int s = 0; s < 4; ++s) {
      bc_[s] = bc[s];
      dir_[s] = dir[s];
    }
  }
  BCType bc_type(BoundaryID side) const override {
    return bc_[static_cast<int>(side)] == 0 ? BCType::Dirichlet : BCType::ZeroFlux;
  }
  double init_f(const Ind& ind) const override { return f0_[ind.i * m_.ny() + ind.j]; }
  void update(double) override {}
  bool dirichlet_vertex_value(BoundaryID side, std::size_t i, std::size_t j, double,
                              double* out) const override {
    const int s = static_cast<int>(side);
    if (bc_[s] != 0 || !dir_[s]) return false;
    *out = (s <= 1) ? dir_[s][j] : dir_[s][i];
    return true;
  }

 private:
  const Mesh& m_;
  const double* f0_;
  int bc_[4];
  const double* dir_[4];
};

std::string g_err;

}  // namespace

extern "C" {

const char* ref_last_error() { return g_err.c_str(); }

// Runs the reference Solver: constructs it (which assembles once from f0, Solver.cc:36-55),
// optionally copies out that first matrix (five diagonals, system order) and RHS, then calls
// update() nsteps times and writes f (alpha-major) to f_out. Returns 0 or -1 (message in
// ref_last_error()).
int ref_run(int nx, int ny, const double* xe, const double* ye, double dt, const int* bc,
            const double* G, const double* Dxx, const double* Dxy, const double* Dyy,
            const double* inv_tau, const double* f0, const double* const* dir, int nsteps,
            double* M5_out, double* R_out, double* f_out) {
  try {
    Grid2D grid(std::vector<double>(xe, xe + nx + 1), std::vector<double>(ye, ye + ny + 1));
    Mesh m(grid, dt);
    ArrayEquation eq(m, G, Dxx, Dxy, Dyy, inv_tau, f0, bc, dir);
    Solver solver(m, &eq);
    const long N = (long)nx * ny;
    if (M5_out) {
      std::memset(M5_out, 0, sizeof(double) * 5 * N);
      const auto& M = solver.M_;
      for (long c = 0; c < N; ++c)
        for (long k = M.colptr[c]; k < M.colptr[c + 1]; ++k) {
          const long r = M.rowind[k];
          int d;
          if (r == c) d = 0;
          else if (c == r - nx) d = 3;
          else if (c == r + nx) d = 4;
          else if (c == r - 1) d = 1;
          else if (c == r + 1) d = 2;
          else { g_err = "unexpected matrix entry outside the 5-point stencil"; return -1; }
          M5_out[d * N + r] = M.vals[k];
        }
    }
    if (R_out)
      for (long K = 0; K < N; ++K) R_out[K] = solver.R_(K);
    for (int s = 0; s < nsteps; ++s) solver.update();
    const auto& f = solver.f();
    for (int i = 0; i < nx; ++i)
      for (int j = 0; j < ny; ++j) f_out[(long)i * ny + j] = f(i, j);
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return -1;
  }
}

}  // extern "C"
