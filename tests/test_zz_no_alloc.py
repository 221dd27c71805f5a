"""sayram_step_noalloc, the entry point for callers that cannot allocate device memory (a host
program whose own memory manager owns the GPU, or one that must not allocate once running).

It is checked through the C-ABI against results that do not come from the library's own
kernels, FP64, for two calls in a row (the second call continues from the first call's output):

* the reference's own Solver (the fixtures of tests/golden/ref_small.npz: f after 1 and 10 steps)
  on ragged, one-wide, non-uniform, all-Dirichlet and all-zero-flux grids;
* the oracle (restated assembly + SuperLU) on a 256 x 256 grid and on a 64 x 1149 grid whose
  padded layout fills the fixed scratch array exactly (round_up((ny+2)*round_up(nx,4), 32) + 64 =
  73728 cells), where an off-by-one in the layout would write past the array;

each to the FP64 parity tolerance of the other tests, 1e-10 in relative L2. nsteps = 0 returns
f_in unchanged. Device buffers for the inputs and outputs are the caller's, here made with torch.
This file is collected last so that a run stopping at the first failure has already run every
other test."""
import ctypes

import numpy as np
import pytest

from conftest import load_small, problem_from
from sayram2d_gb300 import cases

pytestmark = pytest.mark.gpu

Z, NAMES = load_small()
FIXTURE_CASES = ["syn_1x5", "syn_5x1", "syn_17x13_nonuniform", "syn_20x33_alldirichlet",
                 "syn_33x20_zeroflux", "lc_9x4", "syn_24x18_rho-0.9"]


def _dev(torch, a):
    return torch.tensor(np.ascontiguousarray(a, dtype=np.float64), device="cuda")


def _device_problem(capi, torch, p):
    keep = {}
    s = capi.sayram_problem()
    s.nx, s.ny, s.dt = p.nx, p.ny, p.dt
    for name in ("x_edges", "y_edges", "G", "Dxx", "Dxy", "Dyy", "inv_tau"):
        keep[name] = _dev(torch, getattr(p, name))
        setattr(s, name, ctypes.cast(keep[name].data_ptr(), capi._dp))
    s.f0 = capi._dp()
    for side in range(4):
        s.bc[side] = p.bc[side]
        if p.dirichlet[side] is None:
            s.dirichlet[side] = capi._dp()
        else:
            keep[f"dir{side}"] = _dev(torch, p.dirichlet[side])
            s.dirichlet[side] = ctypes.cast(keep[f"dir{side}"].data_ptr(), capi._dp)
    return s, keep


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _two_calls(capi, torch, p, n1, n2):
    """Two calls in a row, the second in place on the first call's output: (f after n1 steps,
    f after n1 + n2 steps, stats of each call)."""
    L = capi.load()
    s, keep = _device_problem(capi, torch, p)
    f_in = _dev(torch, p.f0)
    f_out = torch.empty_like(f_in)
    st1, st2 = capi.sayram_stats(), capi.sayram_stats()
    torch.cuda.synchronize()
    rc = L.sayram_step_noalloc(ctypes.byref(s), None, n1, f_in.data_ptr(), f_out.data_ptr(), None, ctypes.byref(st1))
    assert rc == capi.OK, capi.last_error()
    got1 = f_out.cpu().numpy().reshape(p.nx, p.ny).copy()
    rc = L.sayram_step_noalloc(ctypes.byref(s), None, n2, f_out.data_ptr(), f_out.data_ptr(), None, ctypes.byref(st2))
    assert rc == capi.OK, capi.last_error()
    got2 = f_out.cpu().numpy().reshape(p.nx, p.ny).copy()
    return got1, got2, st1, st2


@pytest.mark.parametrize("name", FIXTURE_CASES)
def test_noalloc_matches_the_reference_solver(capi, name):
    torch = pytest.importorskip("torch")
    p = problem_from(Z, name)
    got1, got10, st1, st2 = _two_calls(capi, torch, p, 1, 9)
    assert st1.steps == 1 and st2.steps == 9 and st1.status == capi.OK and st2.status == capi.OK
    assert rel(got1, Z[f"{name}/f1"]) <= 1e-10, rel(got1, Z[f"{name}/f1"])
    assert rel(got10, Z[f"{name}/f10"]) <= 1e-10, rel(got10, Z[f"{name}/f10"])
    assert got10.min() >= 0.0 and st2.min_f >= 0.0


@pytest.mark.parametrize("nx,ny", [(256, 256), (64, 1149)])
def test_noalloc_matches_the_oracle_up_to_the_scratch_limit(capi, oracle, nx, ny):
    torch = pytest.importorskip("torch")
    pitch = (nx + 3) // 4 * 4
    padded = ((ny + 2) * pitch + 31) // 32 * 32 + 64
    assert padded <= 73728
    if (nx, ny) == (64, 1149):
        assert padded == 73728  # the layout fills the scratch array exactly
    p = cases.synthetic_problem(nx, ny, 1e-2, seed=31 + nx, tau=0.7)
    got1, got2, st1, st2 = _two_calls(capi, torch, p, 2, 2)
    ref1 = oracle.step(p, None, 2, solver="splu")
    ref2 = oracle.step(p, ref1, 2, solver="splu")
    assert rel(got1, ref1) <= 1e-10, rel(got1, ref1)
    assert rel(got2, ref2) <= 1e-10, rel(got2, ref2)
    assert got2.min() >= 0.0 and st1.status == capi.OK and st2.status == capi.OK


def test_noalloc_zero_steps_returns_the_input(capi):
    torch = pytest.importorskip("torch")
    L = capi.load()
    p = cases.synthetic_problem(40, 30, 1e-2, seed=23)
    s, keep = _device_problem(capi, torch, p)
    f_in = _dev(torch, p.f0)
    f_out = torch.full_like(f_in, -1.0)
    st = capi.sayram_stats()
    rc = L.sayram_step_noalloc(ctypes.byref(s), None, 0, f_in.data_ptr(), f_out.data_ptr(), None, ctypes.byref(st))
    assert rc == capi.OK, capi.last_error()
    np.testing.assert_array_equal(f_out.cpu().numpy().reshape(p.nx, p.ny), p.f0)
    assert st.steps == 0 and st.status == capi.OK


def test_noalloc_rejects_grids_beyond_its_scratch(capi):
    torch = pytest.importorskip("torch")
    L = capi.load()
    p = cases.synthetic_problem(40, 30, 1e-2, seed=22)
    s, keep = _device_problem(capi, torch, p)
    f = _dev(torch, p.f0)
    for nx, ny in ((300, 300), (64, 1150)):  # 64 x 1150 is one row past the exact fit
        s.nx, s.ny = nx, ny  # rejected before any array is read
        rc = L.sayram_step_noalloc(ctypes.byref(s), None, 1, f.data_ptr(), f.data_ptr(), None, None)
        assert rc == capi.ERR_ARG
        assert "exceeds the fixed scratch" in capi.last_error()
