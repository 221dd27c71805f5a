"""The C++ drop-in (sayram-2d_gb300/host/Solver.h).

* CPU: it compiles against the reference's unmodified Mesh/Equation headers and links the C-ABI
  library; without a GPU its constructor fails loudly with std::runtime_error (no CPU fallback).
  Needs the reference tree (skipped where it is absent).
* GPU: compiled against project-written stand-ins of the Mesh/Equation interfaces
  (tests/dropin/), it steps the reference's own run configurations through update() -- the
  per-step eq.update(t) and Dirichlet re-upload, and the lazily refreshed host mirror f() -- and
  matches the reference Solver's f at every save (FP64 <= 1e-10, double-word <= 1e-8)."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, reference_tree

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


def _link(capi):
    libdir = os.path.dirname(capi.lib_path())
    return ["-L", libdir, "-lsayram_gpu", f"-Wl,-rpath,{libdir}"]


def test_dropin_compiles_against_reference_headers_and_fails_loudly_without_gpu(capi, tmp_path):
    ref = reference_tree()
    if ref is None:
        pytest.skip("reference tree not present")
    src_dir = os.path.join(ref, "source")
    try:
        import torch

        if torch.cuda.is_available():
            pytest.skip("a GPU is present: the no-GPU failure path cannot be observed")
    except ImportError:
        pass
    src = tmp_path / "dropin_main.cc"
    src.write_text(PROGRAM)
    exe = tmp_path / "dropin"
    cmd = ["g++", "-std=c++17", "-O1", "-w",
           "-I", os.path.join(ROOT, "sayram-2d_gb300", "host"), "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(ROOT, "oracle", "ref_shim"), "-I", src_dir, "-I", os.path.join(src_dir, "Cases"),
           str(src), os.path.join(src_dir, "Mesh.cc"), *_link(capi), "-o", str(exe)]
    subprocess.run(cmd, check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    # this container has no GPU: the constructor must throw, not fall back to the CPU
    assert out.returncode == 3, out.stdout + out.stderr
    assert "runtime_error: sayram_create" in out.stdout


def _build_fixture_driver(capi, tmp_path):
    exe = tmp_path / "dropin_fixture"
    here = os.path.join(ROOT, "tests", "dropin")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-I", here,
           "-I", os.path.join(ROOT, "sayram-2d_gb300", "host"), "-I", os.path.join(ROOT, "include"),
           os.path.join(here, "fixture_main.cc"), *_link(capi), "-o", str(exe)]
    subprocess.run(cmd, check=True)
    return exe


def _write_case(path, p):
    parts = [np.array([p.nx, p.ny, p.dt, *p.bc], dtype=np.float64), p.x_edges, p.y_edges,
             p.G, p.Dxx, p.Dxy, p.Dyy, p.inv_tau, p.f0]
    parts += [p.dirichlet[s] for s in range(4) if p.dirichlet[s] is not None]
    with open(path, "wb") as fh:
        for a in parts:
            fh.write(np.ascontiguousarray(a, dtype=np.float64).tobytes())


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["ay", "lc"])
@pytest.mark.parametrize("prec", [0, 2])
def test_dropin_steps_the_reference_runs_on_the_gpu(capi, tmp_path, name, prec):
    from conftest import ay80_problem

    p, saved = ay80_problem(name)
    exe = _build_fixture_driver(capi, tmp_path)
    case, outp = tmp_path / "case.bin", tmp_path / "out.bin"
    _write_case(case, p)
    nsteps, every = 250, 50
    out = subprocess.run([str(exe), str(case), str(outp), str(nsteps), str(every), str(prec)],
                         capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stdout + out.stderr
    ndir = sum(len(d) for d in p.dirichlet if d is not None)
    assert f"updates={nsteps}" in out.stdout and f"dirichlet_reads_per_step={ndir}" in out.stdout, out.stdout
    f = np.fromfile(outp, dtype=np.float64).reshape(nsteps // every, p.nx, p.ny)
    tol = 1e-10 if prec == 0 else 1e-8
    for k in range(nsteps // every):
        ref = saved[(k + 1) * every]
        err = float(np.linalg.norm(f[k] - ref) / np.linalg.norm(ref))
        assert err <= tol, (name, prec, (k + 1) * every, err)
        assert f[k].min() >= 0.0
