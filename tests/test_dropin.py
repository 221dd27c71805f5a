"""The C++ drop-in (sayram-2d_gb300/host/Solver.h) compiles against the reference's unmodified
Mesh/Equation headers and links the C-ABI library. Without a GPU its constructor must fail
loudly with std::runtime_error (no CPU fallback). CPU only; needs the reference sources."""
import os
import subprocess

import pytest

from conftest import ROOT

REF = "/root/reference/source"

PROGRAM = r'''
#include <cmath>
#include <cstdio>
#include "Solver.h"

class TestEq : public Equation {
 public:
  explicit TestEq(const Mesh& m) : Equation(m), m_(m) {
    for (std::size_t i = 0; i < m.nx(); ++i)
      for (std::size_t j = 0; j < m.ny(); ++j) {
        G_(i, j) = 1.0 + 0.1 * i;
        Dxx_(i, j) = 1e-3; Dyy_(i, j) = 2e-3; Dxy_(i, j) = 5e-4;
      }
  }
  BCType bc_type(BoundaryID s) const override {
    return s == BoundaryID::XMAX ? BCType::ZeroFlux : BCType::Dirichlet;
  }
  double init_f(const Ind& ind) const override { return 1.0 + 0.01 * ind.j; }
  void update(double) override {}
  bool dirichlet_vertex_value(BoundaryID s, std::size_t, std::size_t, double, double* v) const override {
    if (s == BoundaryID::XMAX) return false;
    *v = 0.0;
    return true;
  }
 private:
  const Mesh& m_;
};

int main() {
  std::vector<double> xe(9), ye(7);
  for (int i = 0; i < 9; ++i) xe[i] = 0.1 * i;
  for (int j = 0; j < 7; ++j) ye[j] = 0.2 * j;
  Grid2D grid(xe, ye);
  Mesh m(grid, 0.01);
  TestEq eq(m);
  try {
    Solver solver(m, &eq);
    for (int k = 0; k < 3; ++k) solver.update();
    double s = 0;
    for (std::size_t i = 0; i < m.nx(); ++i)
      for (std::size_t j = 0; j < m.ny(); ++j) s += solver.f({i, j});
    std::printf("ok t=%g sum=%.17g\n", solver.t(), s);
    return 0;
  } catch (const std::runtime_error& e) {
    std::printf("runtime_error: %s\n", e.what());
    return 3;
  }
}
'''


@pytest.mark.skipif(not os.path.isdir(REF), reason="reference sources not present")
def test_dropin_compiles_against_reference_headers_and_fails_loudly_without_gpu(capi, tmp_path):
    src = tmp_path / "dropin_main.cc"
    src.write_text(PROGRAM)
    exe = tmp_path / "dropin"
    libdir = os.path.dirname(capi.lib_path())
    cmd = ["g++", "-std=c++17", "-O1", "-w",
           "-I", os.path.join(ROOT, "sayram-2d_gb300", "host"), "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(ROOT, "oracle", "ref_shim"), "-I", REF, "-I", os.path.join(REF, "Cases"),
           str(src), os.path.join(REF, "Mesh.cc"), "-L", libdir, "-lsayram_gpu", f"-Wl,-rpath,{libdir}",
           "-o", str(exe)]
    subprocess.run(cmd, check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    # this container has no GPU: the constructor must throw, not fall back to the CPU
    assert out.returncode == 3, out.stdout + out.stderr
    assert "runtime_error: sayram_create" in out.stdout
