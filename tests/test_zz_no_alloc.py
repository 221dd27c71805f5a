"""sayram_step_noalloc, the entry point for callers that cannot allocate device memory (a host
program whose own memory manager owns the GPU, or one that must not allocate once running).

It is checked through the C-ABI against the ordinary entry point (sayram_create + sayram_step,
which allocates its own buffers) on the same problem, FP64, for two calls in a row: the second
call continues from the first call's output. Device buffers for the inputs and outputs are the
caller's, here made with torch. Both paths run the same FP64 kernels; the allocating path starts
the second call's solves from a time extrapolation it keeps between calls, so the two agree to
the FP64 parity tolerance of the other tests, 1e-10 in relative L2. This file is collected last
so that a run stopping at the first failure has already run every other test."""
import ctypes

import numpy as np
import pytest

from sayram2d_gb300 import cases

pytestmark = pytest.mark.gpu


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


def test_noalloc_matches_allocating_entry_point(capi):
    torch = pytest.importorskip("torch")
    L = capi.load()
    p = cases.synthetic_problem(96, 80, 1e-2, seed=21, tau=0.5)
    s, keep = _device_problem(capi, torch, p)
    f_in = _dev(torch, p.f0)
    f_out = torch.empty_like(f_in)
    st = capi.sayram_stats()
    torch.cuda.synchronize()
    # first call: f0 -> f_out (3 steps)
    rc = L.sayram_step_noalloc(ctypes.byref(s), None, 3, f_in.data_ptr(), f_out.data_ptr(), None, ctypes.byref(st))
    assert rc == capi.OK, capi.last_error()
    got1 = f_out.cpu().numpy().reshape(p.nx, p.ny)
    assert st.steps == 3 and st.status == capi.OK and st.min_f >= 0.0
    # second call continues from the first call's output, in place
    rc = L.sayram_step_noalloc(ctypes.byref(s), None, 3, f_out.data_ptr(), f_out.data_ptr(), None, ctypes.byref(st))
    assert rc == capi.OK, capi.last_error()
    got2 = f_out.cpu().numpy().reshape(p.nx, p.ny)
    assert st.steps == 3 and st.min_f >= 0.0
    ref = capi.Solver(p, precision=capi.FP64)
    ref.step(3)
    ref1 = ref.f()
    ref.step(3)
    ref2 = ref.f()
    ref.close()
    assert rel(got1, ref1) <= 1e-10, rel(got1, ref1)
    assert rel(got2, ref2) <= 1e-10, rel(got2, ref2)
    assert got2.min() >= 0.0


def test_noalloc_rejects_grids_beyond_its_scratch(capi):
    torch = pytest.importorskip("torch")
    L = capi.load()
    p = cases.synthetic_problem(40, 30, 1e-2, seed=22)
    s, keep = _device_problem(capi, torch, p)
    f = _dev(torch, p.f0)
    s.nx, s.ny = 300, 300  # rejected before any array is read
    rc = L.sayram_step_noalloc(ctypes.byref(s), None, 1, f.data_ptr(), f.data_ptr(), None, None)
    assert rc == capi.ERR_ARG
    assert "exceeds the fixed scratch" in capi.last_error()
