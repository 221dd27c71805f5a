// ref_case_harness.cc -- TEST INFRASTRUCTURE. Runs the reference's own Albert_Young and
// Albert_Young_LC cases (Sayram-2D source/Cases/Albert_Young{,_LC,_IO}.cc, compiled unmodified
// against the shim headers in ref_shim/) on a grid and a D table supplied by the tests, and
// returns what a Solver would read from them: G, Dxx, Dxy, Dyy, inv_tau, init_f, the BC types
// and the Dirichlet vertex values. The D table reaches Albert_Young_IO::read_D through the shim's
// load_hdf5 registry, under the names read_D asks for ("D/<dID>.h5": /alpha0, /E, /Daa, /Dap,
// /Dpp).
//
// Parameters' constructor (Parameters.cc) parses an ini file and creates output directories; the
// cases only read logEmin() and dID() from it, so this harness defines the constructor itself and
// fills those members from the call's arguments.
#include <cmath>
#include <cstring>
#include <exception>
#include <string>
#include <vector>

#include "common.h"
#include "Grid2D.h"
#include "Mesh.h"
#include "Parameters.h"
#include "Albert_Young.h"
#include "Albert_Young_LC.h"

namespace {
struct HarnessParams {
  double Emin = 0.2, Emax = 5.0;
  std::string dID = "harness";
} g_par;
std::string g_err;
}  // namespace

Parameters::Parameters(int, char**) {
  inp_file_ = "harness";
  run_id_ = "harness";
  Emin_ = g_par.Emin;
  Emax_ = g_par.Emax;
  logEmin_ = log(Emin_);
  logEmax_ = log(Emax_);
  dID_ = g_par.dID;
}

extern "C" const char* ref_case_last_error() { return g_err.c_str(); }

// which: 0 = Albert_Young, 1 = Albert_Young_LC. Fields out are (nx, ny) alpha-major; bc[4] is
// 0 (Dirichlet) / 1 (zero flux) for XMIN, XMAX, YMIN, YMAX; dir receives, per side, ny+1 (x sides)
// or nx+1 (y sides) vertex values at offsets 0, ny+1, 2(ny+1), 2(ny+1)+nx+1.
extern "C" int ref_case(int which, int nx, int ny, const double* xe, const double* ye, double dt, double Emin,
                        double Emax, int na, int ne, const double* alpha0_deg, const double* E, const double* Daa,
                        const double* Dap, const double* Dpp, double* G, double* Dxx, double* Dxy, double* Dyy,
                        double* inv_tau, double* f0, int* bc, double* dir) {
  try {
    g_par.Emin = Emin;
    g_par.Emax = Emax;
    auto& reg = shim_h5::registry();
    reg.clear();
    const std::string file = "D/" + g_par.dID + ".h5";
    reg[file + ":/alpha0"] = {std::vector<double>(alpha0_deg, alpha0_deg + na), (std::size_t)na, 1};
    reg[file + ":/E"] = {std::vector<double>(E, E + ne), (std::size_t)ne, 1};
    const std::size_t nt = (std::size_t)na * ne;
    reg[file + ":/Daa"] = {std::vector<double>(Daa, Daa + nt), (std::size_t)na, (std::size_t)ne};
    reg[file + ":/Dap"] = {std::vector<double>(Dap, Dap + nt), (std::size_t)na, (std::size_t)ne};
    reg[file + ":/Dpp"] = {std::vector<double>(Dpp, Dpp + nt), (std::size_t)na, (std::size_t)ne};
    char arg0[] = "harness";
    char* argv[] = {arg0, nullptr};
    Parameters paras(1, argv);
    Grid2D grid(std::vector<double>(xe, xe + nx + 1), std::vector<double>(ye, ye + ny + 1));
    Mesh m(grid, dt);
    Albert_Young* ay = nullptr;
    Albert_Young_LC* lc = nullptr;
    Equation* eq;
    if (which == 0)
      eq = ay = new Albert_Young(paras, m);
    else
      eq = lc = new Albert_Young_LC(paras, m);
    for (std::size_t i = 0; i < (std::size_t)nx; ++i)
      for (std::size_t j = 0; j < (std::size_t)ny; ++j) {
        const std::size_t c = i * ny + j;
        const Ind ind{i, j};
        G[c] = eq->G(ind);
        Dxx[c] = eq->Dxx(ind);
        Dxy[c] = eq->Dxy(ind);
        Dyy[c] = eq->Dyy(ind);
        inv_tau[c] = eq->inv_tau(ind);
        f0[c] = eq->init_f(ind);
      }
    const BoundaryID sides[4] = {BoundaryID::XMIN, BoundaryID::XMAX, BoundaryID::YMIN, BoundaryID::YMAX};
    std::size_t off = 0;
    for (int s = 0; s < 4; ++s) {
      bc[s] = eq->bc_type(sides[s]) == BCType::Dirichlet ? 0 : 1;
      const std::size_t n = (s <= 1) ? ny + 1 : nx + 1;
      for (std::size_t k = 0; k < n; ++k) {
        const std::size_t i = (s == 0) ? 0 : (s == 1) ? nx : k;
        const std::size_t j = (s <= 1) ? k : (s == 2) ? 0 : ny;
        double v = 0.0;
        dir[off + k] = eq->dirichlet_vertex_value(sides[s], i, j, 0.0, &v) ? v : 0.0;
      }
      off += n;
    }
    delete ay;
    delete lc;
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return 1;
  }
}
