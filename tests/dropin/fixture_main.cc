// TEST INFRASTRUCTURE: host/Solver.h (the C++ drop-in) stepped through update() like main.cc's
// time loop (main.cc:77-85). The Equation serves a case read from a raw binary file written by
// tests/test_dropin.py: nx, ny, dt, bc[4], edges, G, Dxx, Dxy, Dyy, inv_tau, f0 (alpha-major) and
// the Dirichlet vertex values per side. update(t) counts its calls, and the Dirichlet values are
// served through dirichlet_vertex_value on every step, so the per-step re-read is exercised.
// Prints f after every `every` steps as raw doubles to the output file.
#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include <vector>

#include "Solver.h"

namespace {
std::vector<double> take(std::FILE* fp, std::size_t n) {
  std::vector<double> v(n);
  if (n && std::fread(v.data(), sizeof(double), n, fp) != n) throw std::runtime_error("short fixture file");
  return v;
}
}  // namespace

class FixtureEq : public Equation {
 public:
  FixtureEq(const Mesh& m, const std::vector<double>* fields, const std::vector<double>* dir, const int* bc)
      : Equation(m), m_(m) {
    Xtensor2d* dst[5] = {&G_, &Dxx_, &Dxy_, &Dyy_, &inv_tau_};
    for (int k = 0; k < 5; ++k)
      for (std::size_t i = 0; i < m.nx(); ++i)
        for (std::size_t j = 0; j < m.ny(); ++j) (*dst[k])(i, j) = fields[k][i * m.ny() + j];
    f0_ = fields[5];
    for (int s = 0; s < 4; ++s) {
      bc_[s] = bc[s];
      dir_[s] = dir[s];
    }
  }
  BCType bc_type(BoundaryID s) const override { return bc_[(int)s] == 0 ? BCType::Dirichlet : BCType::ZeroFlux; }
  double init_f(const Ind& k) const override { return f0_[k.i * m_.ny() + k.j]; }
  void update(double) override { ++updates; }
  bool dirichlet_vertex_value(BoundaryID s, std::size_t i, std::size_t j, double, double* v) const override {
    const int side = (int)s;
    if (bc_[side] != 0) return false;
    ++dirichlet_reads;
    *v = dir_[side][side <= 1 ? j : i];
    return true;
  }
  long updates = 0;
  mutable long dirichlet_reads = 0;

 private:
  const Mesh& m_;
  std::vector<double> f0_, dir_[4];
  int bc_[4];
};

int main(int argc, char** argv) {
  if (argc != 6) {
    std::fprintf(stderr, "usage: %s case.bin out.bin nsteps every precision\n", argv[0]);
    return 2;
  }
  try {
    std::FILE* fp = std::fopen(argv[1], "rb");
    if (!fp) throw std::runtime_error("cannot open the case file");
    const std::vector<double> head = take(fp, 7);
    const std::size_t nx = (std::size_t)head[0], ny = (std::size_t)head[1];
    const double dt = head[2];
    int bc[4];
    for (int s = 0; s < 4; ++s) bc[s] = (int)head[3 + s];
    const std::vector<double> xe = take(fp, nx + 1), ye = take(fp, ny + 1);
    std::vector<double> fields[6];
    for (auto& f : fields) f = take(fp, nx * ny);
    std::vector<double> dir[4];
    for (int s = 0; s < 4; ++s) dir[s] = take(fp, bc[s] == 0 ? ((s <= 1) ? ny + 1 : nx + 1) : 0);
    std::fclose(fp);
    Mesh m(xe, ye, dt);
    FixtureEq eq(m, fields, dir, bc);
    const int nsteps = std::atoi(argv[3]), every = std::atoi(argv[4]), prec = std::atoi(argv[5]);
    Solver solver(m, &eq, prec);
    std::FILE* out = std::fopen(argv[2], "wb");
    if (!out) throw std::runtime_error("cannot open the output file");
    const long reads0 = eq.dirichlet_reads;
    for (int k = 1; k <= nsteps; ++k) {
      solver.update();
      if (k % every == 0) {
        const Xtensor2d& f = solver.f();
        for (std::size_t i = 0; i < nx; ++i)
          for (std::size_t j = 0; j < ny; ++j) {
            const double v = f(i, j);
            std::fwrite(&v, sizeof(double), 1, out);
          }
      }
    }
    std::fclose(out);
    std::printf("ok t=%.17g updates=%ld dirichlet_reads_per_step=%ld f00=%.17g\n", solver.t(), eq.updates,
                (eq.dirichlet_reads - reads0) / (nsteps > 0 ? nsteps : 1), solver.f({0, 0}));
    return 0;
  } catch (const std::runtime_error& e) {
    std::printf("runtime_error: %s\n", e.what());
    return 3;
  }
}
