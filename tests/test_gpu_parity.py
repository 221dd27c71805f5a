"""GPU parity: the CUDA path through the C-ABI against the reference-generated fixtures and the
oracle. Tolerances: the plain FP64 drop-in must match the reference solution to a relative L2
error <= 1e-10 and stay non-negative; the FP32+FP64-refinement path to <= 1e-8.

Matrix entries: the GPU evaluates the reference's formulas with fused multiply-adds and a
reciprocal of (f + eps). Where f is about eps, B+/(f + eps) magnifies the rounding of a nearly
cancelling a_sigma = aA*fA + aB*fB (the reference compiled with FMA contraction, the default of
its own clang build, moves such entries too). Each entry is therefore held to 1e-12 of its
forward-error scale: the same formula evaluated on the magnitudes of its terms (oracle
assemble_bound), about 4500 units in the last place of that scale."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, c0_problem, load_small, problem_from
from sayram2d_gb300 import cases

pytestmark = pytest.mark.gpu

Z, NAMES = load_small()
TOL64, TOL32 = 1e-10, 1e-8


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("name", NAMES)
def test_assembly_matches_reference(capi, oracle, name):
    p = problem_from(Z, name)
    ref, Rref = Z[f"{name}/M5"], Z[f"{name}/R"]
    M5o, _, bound = oracle.assemble_bound(p, p.f0)
    assert np.array_equal(M5o, ref)
    for prec in (capi.FP64, capi.FP32_REFINE, capi.FP32_REFINE_DW):
        s = capi.Solver(p, precision=prec)
        M5, R = s.export_system(0)
        s.close()
        err = np.abs(M5 - ref)
        assert (err <= 1e-12 * bound).all(), (name, prec, (err / np.maximum(bound, 1e-300)).max())
        assert np.allclose(R, Rref, rtol=1e-13, atol=1e-300), name


@pytest.mark.parametrize("name", NAMES)
@pytest.mark.parametrize("prec", [0, 1, 2])
def test_steps_match_reference(capi, name, prec):
    p = problem_from(Z, name)
    s = capi.Solver(p, precision=prec)
    tol = TOL64 if prec == capi.FP64 else TOL32
    s.update()
    f1 = s.f()
    assert rel(f1, Z[f"{name}/f1"]) <= tol, (name, rel(f1, Z[f"{name}/f1"]))
    for _ in range(9):
        s.update()
    f10 = s.f()
    st = s.get_stats()
    s.close()
    assert rel(f10, Z[f"{name}/f10"]) <= tol, (name, rel(f10, Z[f"{name}/f10"]), st)
    assert f10.min() >= 0.0 and st["min_f"] >= 0.0
    assert st["steps"] == 10 and abs(st["t"] - 10 * p.dt) < 1e-12
    assert st["rel_residual"] <= (1e-12 if prec == capi.FP64 else 1e-10)
    assert st["mass_drift"] <= 1e-8


def test_config0_full_run_fp64(capi):
    """Config 0: 90 x 90, dt = 1e-3, 1000 steps, against the reference's own result."""
    z = np.load(os.path.join(GOLDEN, "ref_c0_90x90.npz"))
    rp, p = c0_problem()
    s = capi.Solver(p, precision=capi.FP64)
    s.step(rp.nsteps)
    f = s.f()
    st = s.get_stats()
    s.close()
    assert rel(f, z[f"f{rp.nsteps}"]) <= TOL64, rel(f, z[f"f{rp.nsteps}"])
    assert f.min() >= 0.0
    assert st["steps"] == rp.nsteps


@pytest.mark.parametrize("prec", [1, 2])
def test_config0_full_run_mixed(capi, prec):
    z = np.load(os.path.join(GOLDEN, "ref_c0_90x90.npz"))
    rp, p = c0_problem()
    s = capi.Solver(p, precision=prec)
    s.step(rp.nsteps)
    f = s.f()
    s.close()
    assert rel(f, z[f"f{rp.nsteps}"]) <= TOL32
    assert f.min() >= 0.0


def test_batch_equals_alone(capi):
    """Each instance advanced inside an uneven batch equals the same instance advanced alone."""
    probs = [problem_from(Z, n) for n in NAMES] + cases.batch_problems(6, seed=5, dt=1e-2, lo=40, hi=90)
    for prec, tol in ((capi.FP64, 1e-12), (capi.FP32_REFINE, 1e-8), (capi.FP32_REFINE_DW, 1e-8)):
        b = capi.Batch(probs, precision=prec)
        b.step(5)
        got = [b.f(k) for k in range(len(probs))]
        b.close()
        for k, p in enumerate(probs):
            s = capi.Solver(p, precision=prec)
            s.step(5)
            alone = s.f()
            s.close()
            assert rel(got[k], alone) <= tol, (prec, k, rel(got[k], alone))


@pytest.mark.parametrize("prec", [1, 2])
def test_batch_vs_oracle(capi, oracle, prec):
    probs = cases.batch_problems(5, seed=11, dt=1e-2, lo=64, hi=100)
    b = capi.Batch(probs, precision=prec)
    b.step(3)
    for k, p in enumerate(probs):
        ref = oracle.step(p, None, 3)
        f = b.f(k)
        assert rel(f, ref) <= TOL32 and f.min() >= 0.0
        st = b.stats(k)
        assert st["mass_drift"] <= 1e-8 and st["rel_residual"] <= 1e-10
    b.close()


@pytest.mark.parametrize("prec", [0, 2])
def test_benchmark_batch_sample_vs_oracle(capi, oracle, prec):
    """The benchmark's batch distribution (nalpha, nE ~ U[64, 256], rho ~ U[-0.9, 0.9], tau
    log-uniform in [0.1, 10] days, dt = 1e-2): 48 instances stepped together 4 times; 8 of them,
    spread over the size range, against the oracle (restated assembly + SuperLU) stepped alone;
    FP64 <= 1e-10, double-word path <= 1e-8; every instance non-negative and mass-conserving."""
    sizes = cases.batch_sizes(48, 2024)
    probs = [cases.batch_instance(k, 2024, 1e-2, sizes[k]) for k in range(48)]
    b = capi.Batch(probs, precision=prec)
    b.step(4)
    tol = TOL64 if prec == 0 else TOL32
    cells = np.array([a * e for a, e in sizes])
    pick = sorted({int(np.argsort(cells)[q]) for q in np.linspace(0, 47, 8).round().astype(int)})
    for k in pick:
        ref = oracle.step(probs[k], None, 4, solver="splu")
        assert rel(b.f(k), ref) <= tol, (prec, k, sizes[k], rel(b.f(k), ref))
    for k in range(48):
        st = b.stats(k)
        assert st["min_f"] >= 0.0 and st["mass_drift"] <= 1e-9 and st["status"] == 0, (k, st)
    b.close()


@pytest.mark.parametrize("prec", [0, 2])
def test_step_host_roundtrip(capi, prec):
    probs = cases.batch_problems(4, seed=2, dt=1e-2, lo=30, hi=70)
    b = capi.Batch(probs, precision=prec)
    fin = np.concatenate([p.f0.ravel() for p in probs])
    fout = np.empty_like(fin)
    b.step_host(2, fin.ctypes.data, fout.ctypes.data)
    off = 0
    for k, p in enumerate(probs):
        n = p.nx * p.ny
        assert np.array_equal(fout[off:off + n].reshape(p.nx, p.ny), b.f(k))
        off += n
    c = capi.Batch(probs, precision=prec)
    c.step(2)
    for k in range(len(probs)):
        assert rel(b.f(k), c.f(k)) <= 1e-12
    b.close()
    c.close()


@pytest.mark.parametrize("prec", [0, 2])
def test_cooperative_solve_equals_separate_kernels(capi, prec):
    """A batch whose chunks fit in one wave of co-resident blocks runs each step's refinement
    loop as one cooperative kernel (grid-wide barriers between the passes); switched off, the
    same loop runs as the graph's (or the host loop's) separate kernels. The states must agree
    bit for bit, and the cooperative form must take far fewer launches."""
    probs = [cases.synthetic_problem(200, 150, 1e-2, 3)] + cases.batch_problems(3, seed=4, dt=1e-2, lo=30, hi=90)
    states, launches = {}, {}
    for coop in (True, False):
        for graph in (1, 0):
            b = capi.Batch(probs, precision=prec, use_graph=graph)
            b.set_coop(coop)
            l0 = b.launches()
            b.step(4)
            launches[(coop, graph)] = b.launches() - l0
            states[(coop, graph)] = [b.f(k) for k in range(len(probs))]
            assert all(b.stats(k)["status"] == 0 for k in range(len(probs)))
            b.close()
    ref = states[(False, 1)]
    for key, fs in states.items():
        for k, (a, c) in enumerate(zip(ref, fs)):
            assert np.array_equal(a, c), (key, k, rel(a, c))
    assert launches[(True, 1)] < launches[(False, 1)] / 3, launches
    assert launches[(True, 0)] < launches[(False, 0)] / 3, launches


def test_layout_transforms_round_like_the_host(capi):
    """The host-buffer step's layout transforms convert double <-> double word with integer
    rounding on the device (dw_from_double_int / dw_to_double_int). A zero-step call round-trips
    a state through both; every value must come back as float64(hi) + float64(lo) with
    hi = float32(v), lo = float32(v - hi), the separately rounded IEEE conversions, bit for bit:
    over 600 decades, signed zeros, float32 subnormals and boundaries, and rounding ties."""
    probs = cases.batch_problems(3, seed=5, dt=1e-2, lo=30, hi=70)
    b = capi.Batch(probs, precision=2)
    n = sum(p.nx * p.ny for p in probs)
    rng = np.random.default_rng(11)
    v = rng.choice([-1.0, 1.0], n) * 10.0 ** rng.uniform(-300, 38, n)
    h = rng.uniform(0.5, 1.0, n).astype(np.float32).astype(np.float64)
    k = np.arange(n)
    # ties of the 24-bit rounding: a float32 value in [0.5, 1) plus exactly half its last place
    v[k % 7 == 1] = (h + 2.0 ** -25)[k % 7 == 1] * 2.0 ** rng.integers(-120, 120, n)[k % 7 == 1]
    v[k % 7 == 2] = np.float64(np.float32(1.1754943508222875e-38)) * rng.uniform(0.5, 2.0, n)[k % 7 == 2]
    v[k % 7 == 3] = 1.401298464324817e-45 * rng.uniform(0.0, 4.0, n)[k % 7 == 3]
    v[k % 97 == 4] = 0.0
    v[k % 97 == 5] = -0.0
    v[k % 97 == 6] = 3.4028234663852886e38
    fin = np.ascontiguousarray(v)
    fout = np.empty_like(fin)
    b.step_host(0, fin.ctypes.data, fout.ctypes.data)
    with np.errstate(over="ignore", under="ignore", invalid="ignore"):
        hi = fin.astype(np.float32)
        lo = (fin - hi.astype(np.float64)).astype(np.float32)
        want = hi.astype(np.float64) + lo.astype(np.float64)
    bad = np.flatnonzero(fout.view(np.uint64) != want.view(np.uint64))
    assert bad.size == 0, (bad.size, fin[bad[:3]], fout[bad[:3]], want[bad[:3]])
    b.close()


@pytest.mark.parametrize("prec", [0, 2])
def test_step_host_forms_equal_device_stepping(capi, prec):
    """Every form of the host-buffer step (state in and out, in only, out only; one to five steps,
    so the first and last steps run split around the copies and the middle ones as whole-step
    graphs) leaves bit for bit the state of the same steps taken on the device."""
    probs = cases.batch_problems(5, seed=31, dt=1e-2, lo=30, hi=90)
    a = capi.Batch(probs, precision=prec)
    b = capi.Batch(probs, precision=prec)
    a.step(1)
    b.step(1)
    n = sum(p.nx * p.ny for p in probs)
    for nsteps, with_in, with_out in ((1, True, True), (2, True, False), (3, False, True), (5, True, True),
                                      (1, False, True), (4, True, True)):
        fin = np.concatenate([a.f(k).ravel() for k in range(len(probs))]) if with_in else None
        fout = np.full(n, np.nan) if with_out else None
        a.step_host(nsteps, fin.ctypes.data if with_in else None, fout.ctypes.data if with_out else None)
        b.step(nsteps)
        want = np.concatenate([b.f(k).ravel() for k in range(len(probs))])
        got = np.concatenate([a.f(k).ravel() for k in range(len(probs))])
        assert np.array_equal(got, want), (nsteps, with_in, with_out)
        if with_out:
            assert np.array_equal(fout, want), (nsteps, with_in, with_out)
        for k in range(len(probs)):
            sa, sb = a.stats(k), b.stats(k)
            assert sa["steps"] == sb["steps"] and sa["min_f"] == sb["min_f"] and sa["mass_drift"] == sb["mass_drift"]
    a.close()
    b.close()


def test_set_f_get_f_and_dirichlet(capi, oracle):
    p = cases.synthetic_problem(20, 15, 1e-2, seed=3)
    s = capi.Solver(p)
    g = np.random.default_rng(0).uniform(0, 1, (20, 15))
    s.set_f(g)
    assert np.array_equal(s.f(), g)
    newv = np.linspace(0.0, 0.5, 21)
    s.set_dirichlet(cases.YMIN, newv)
    p2 = cases.synthetic_problem(20, 15, 1e-2, seed=3)
    p2.dirichlet[cases.YMIN] = newv
    p2.f0 = g
    s.update()
    assert rel(s.f(), oracle.step(p2, g, 1)) <= TOL64
    with pytest.raises(RuntimeError, match="not Dirichlet"):
        s.set_dirichlet(cases.XMAX, np.zeros(16))
    s.close()


@pytest.mark.parametrize("prec", [0, 2])
def test_time_dependent_coefficients(capi, oracle, prec):
    """Equation::update with new G, D and 1/tau between steps (sayram_set_coeffs, the path of
    Solver.h's time_dependent_coeffs): the steps after the change match the oracle stepping the
    changed problem from the same state, in a single instance and inside a batch."""
    import dataclasses

    p = cases.synthetic_problem(40, 30, 1e-2, seed=8)
    rng = np.random.default_rng(3)
    scale = rng.uniform(0.5, 2.0, size=(40, 30))
    q = dataclasses.replace(p, G=p.G * 1.1, Dxx=p.Dxx * scale, Dxy=p.Dxy * 0.5 * scale, Dyy=p.Dyy * scale[::-1, ::-1],
                            inv_tau=p.inv_tau + 0.3)
    tol = TOL64 if prec == capi.FP64 else TOL32
    s = capi.Solver(p, precision=prec)
    s.step(2)
    mid = s.f()
    s.set_coeffs(q.G, q.Dxx, q.Dxy, q.Dyy, q.inv_tau)
    s.step(3)
    ref = oracle.step(q, mid, 3)
    assert rel(s.f(), ref) <= tol and s.f().min() >= 0.0
    s.close()
    others = cases.batch_problems(3, seed=9, dt=1e-2, lo=20, hi=50)
    b = capi.Batch([others[0], p, others[1]], precision=prec)
    b.step(2)
    mid_b = b.f(1)
    b.set_coeffs(1, q.G, q.Dxx, q.Dxy, q.Dyy, q.inv_tau)
    b.step(3)
    assert rel(b.f(1), oracle.step(q, mid_b, 3)) <= tol
    assert rel(b.f(0), oracle.step(others[0], None, 5)) <= tol  # the neighbours are untouched
    b.close()


def test_not_converged_is_reported_not_hidden(capi):
    """A forced non-convergence (one Krylov iteration, two residual checks) returns
    NOT_CONVERGED but the state still advances and stays non-negative."""
    p = cases.synthetic_problem(64, 64, 1e-2, seed=4)
    s = capi.Solver(p, precision=capi.FP64, max_iters=1, max_refine=2)
    rc = s.step(1, allow_not_converged=True)
    assert rc == capi.ERR_NOT_CONVERGED
    st = s.get_stats()
    assert st["status"] == capi.ERR_NOT_CONVERGED and st["steps"] == 1
    assert s.f().min() >= 0.0
    s.close()


def test_large_grid_properties(capi, oracle):
    """512 x 512, dt = 1e-2: two steps against SuperLU, plus conservation and positivity."""
    p = cases.synthetic_problem(512, 512, 1e-2, seed=5)
    s = capi.Solver(p, precision=capi.FP64)
    s.step(2)
    f = s.f()
    st = s.get_stats()
    s.close()
    ref = oracle.step(p, None, 2, solver="splu")
    assert rel(f, ref) <= TOL64, rel(f, ref)
    assert f.min() >= 0.0 and st["mass_drift"] <= 1e-9


@pytest.mark.parametrize("name", ["ay", "lc"])
@pytest.mark.parametrize("prec", [0, 2])
def test_reference_run_configuration_ay80(capi, prec, name):
    """The reference's own run configurations (p.ini: Albert_Young; p_AlbertYoungLC.ini:
    Albert_Young_LC; 80 x 80, T = 1 day in 500 steps) with the fields the reference's case built
    from its own D table, against the reference Solver's f at every save (every 50 steps)."""
    from conftest import ay80_problem

    p, saved = ay80_problem(name)
    tol = TOL64 if prec == capi.FP64 else TOL32
    s = capi.Solver(p, precision=prec)
    done = 0
    for n in sorted(saved):
        s.step(n - done)
        done = n
        f = s.f()
        assert rel(f, saved[n]) <= tol, (prec, n, rel(f, saved[n]))
        assert f.min() >= 0.0
    s.close()


@pytest.mark.parametrize("name,ini", [("ay", "albert_young_80x80.ini"), ("lc", "albert_young_lc_80x80.ini")])
@pytest.mark.parametrize("prec", ["fp64", "fp32_refine_dw"])
def test_run_reference_ini_with_its_d_table(capi, tmp_path, prec, name, ini):
    """main.cc end to end on the reference's run files (the same keys as its p.ini and
    p_AlbertYoungLC.ini): run.run reads the ini, selects Albert_Young / Albert_Young_LC, reads
    D/AlbertYoung_chorus.h5 (written here from the reference's table values with the library's
    own writer), interpolates D on the device and writes /f/0 .. /f/10; every save is compared with
    the reference Solver's f at that step (FP64 drop-in <= 1e-10, double-word path <= 1e-8)."""
    import shutil

    from conftest import ay80_problem, ay80_table
    from sayram2d_gb300 import run

    p, saved = ay80_problem(name)
    t = ay80_table()
    os.makedirs(tmp_path / "D")
    with capi.H5File(str(tmp_path / "D" / "AlbertYoung_chorus.h5")) as h5:
        h5.write("/alpha0", t.alpha0_deg)
        h5.write("/E", t.E)
        h5.write("/Daa", t.Daa)
        h5.write("/Dap", t.Dap)
        h5.write("/Dpp", t.Dpp)
    src = tmp_path / ini
    shutil.copyfile(os.path.join(ROOT, "sayram-2d_gb300", "configs", ini), src)
    path = run.run(str(src), root=str(tmp_path), precision=prec)
    tol = TOL64 if prec == "fp64" else TOL32
    f0 = capi.h5_read(path, "/f/0")
    assert np.allclose(f0, p.f0, rtol=1e-13, atol=0.0)
    for k, n in enumerate(sorted(saved), start=1):
        f = capi.h5_read(path, f"/f/{k}")
        assert rel(f, saved[n]) <= tol, (prec, name, k, rel(f, saved[n]))
        assert f.min() >= 0.0
    np.testing.assert_array_equal(capi.h5_read(path, "/t"), np.linspace(0.0, 1.0, 11))


def _c1_close(z, pre, f, tol):
    sub = f[::8, ::8]
    assert rel(sub, z[pre + "_sub"]) <= tol, (pre, rel(sub, z[pre + "_sub"]))
    assert rel(f.sum(axis=1), z[pre + "_rows"]) <= tol, (pre, "rows")
    assert rel(f.sum(axis=0), z[pre + "_cols"]) <= tol, (pre, "cols")


def test_config1_prefix_against_superlu_fixture(capi):
    """Config 1 at full size (1024 x 1024, dt = 1e-2): 1 and 10 steps of the FP64 drop-in and of
    the double-word path against the fixture made with the restated assembly and SuperLU
    (strided sample of f, row and column sums, sum of squares)."""
    z = np.load(os.path.join(GOLDEN, "ref_c1_1024_prefix.npz"))
    n = int(z["nsteps"][0])
    p = cases.synthetic_problem(1024, 1024, 1e-2, seed=11)
    for prec, tol in ((capi.FP64, TOL64), (capi.FP32_REFINE_DW, TOL32)):
        s = capi.Solver(p, precision=prec)
        s.step(1)
        _c1_close(z, "f1", s.f(), tol)
        s.step(n - 1)
        f = s.f()
        s.close()
        _c1_close(z, "fN", f, tol)
        assert abs(float((f * f).sum()) - z["fN_ssq"][0]) <= 2 * tol * z["fN_ssq"][0]
        assert f.min() >= 0.0


@pytest.mark.parametrize("prec", [0, 2])
def test_config1_all_500_steps_against_tight_oracle(capi, prec):
    """Config 1 over its whole run (1024 x 1024, dt = 1e-2, 500 steps) against the tight-residual
    oracle (restated assembly, alpha-line-preconditioned BiCGSTAB inside refinement with
    extended-precision residuals; it agrees with the SuperLU direct solve over the first 10
    steps): a strided sample of f, its row and column sums and its sum of squares at steps 10,
    100, 250 and 500, FP64 drop-in <= 1e-10, double-word path <= 1e-8, min f >= 0."""
    path = os.path.join(GOLDEN, "ref_c1_1024_full.npz")
    if not os.path.exists(path):
        pytest.skip("ref_c1_1024_full.npz not generated (tests/golden/make_golden.py config1_full)")
    z = np.load(path)
    p = cases.synthetic_problem(1024, 1024, 1e-2, seed=11)
    tol = TOL64 if prec == 0 else TOL32
    s = capi.Solver(p, precision=prec)
    done = 0
    for n in [int(v) for v in z["saves"]]:
        s.step(n - done)
        done = n
        f = s.f()
        assert f.min() >= 0.0
        _c1_close(z, f"f{n}", f, tol)
        ssq = float((f * f).sum())
        assert abs(ssq - z[f"f{n}_ssq"][0]) <= 2 * tol * z[f"f{n}_ssq"][0], (n, ssq)
    st = s.get_stats()
    s.close()
    assert st["steps"] == 500 and st["status"] == 0


def test_config1_size_1024(capi, oracle):
    """The single-instance configuration at full size (1024 x 1024, dt = 1e-2): one step of the
    FP64 path against SuperLU, then size-independent properties over further steps -- the
    double-word path within 1e-8 of the FP64 path, conservation, positivity, residual."""
    p = cases.synthetic_problem(1024, 1024, 1e-2, seed=11)
    s64 = capi.Solver(p, precision=capi.FP64)
    s64.step(1)
    ref = oracle.step(p, None, 1, solver="splu")
    assert rel(s64.f(), ref) <= TOL64, rel(s64.f(), ref)
    sdw = capi.Solver(p, precision=capi.FP32_REFINE_DW)
    sdw.step(1)
    s64.step(3)
    sdw.step(3)
    f64, fdw = s64.f(), sdw.f()
    assert rel(fdw, f64) <= TOL32, rel(fdw, f64)
    for st, tol in ((s64.get_stats(), 1e-12), (sdw.get_stats(), 1e-11)):
        assert st["rel_residual"] <= tol and st["mass_drift"] <= 1e-9 and st["status"] == 0
    assert f64.min() >= 0.0 and fdw.min() >= 0.0
    s64.close()
    sdw.close()


def test_tiny_magnitudes(capi, oracle):
    """f0 and the Dirichlet values scaled by 2^-100 (~1e-30): the FP32 inner solves see residuals
    scaled by a power of two near max|R| (no FP32 underflow), so every mode still matches the
    oracle on this problem."""
    q = cases.synthetic_problem(48, 40, 1e-2, seed=6)
    sc = 2.0 ** -100
    q.f0 = q.f0 * sc
    q.dirichlet = [None if d is None else d * sc for d in q.dirichlet]
    ref = oracle.step(q, None, 3)
    for prec, tol in ((capi.FP64, TOL64), (capi.FP32_REFINE, TOL32), (capi.FP32_REFINE_DW, TOL32)):
        c = capi.Solver(q, precision=prec)
        c.step(3)
        fc = c.f()
        st = c.get_stats()
        c.close()
        assert rel(fc, ref) <= tol, (prec, rel(fc, ref))
        assert fc.min() >= 0.0


@pytest.mark.parametrize("prec", [0, 1, 2])
def test_graph_equals_host_loop(capi, prec):
    """The per-step CUDA graph (device-side WHILE loops) runs the same kernels in the same order
    as the host-driven loop, so the results are identical."""
    probs = cases.batch_problems(5, seed=9, dt=1e-2, lo=20, hi=90)
    g = capi.Batch(probs, precision=prec, use_graph=1)
    h = capi.Batch(probs, precision=prec, use_graph=0)
    g.step(4)
    h.step(4)
    for k in range(len(probs)):
        assert np.array_equal(g.f(k), h.f(k)), (prec, k, rel(g.f(k), h.f(k)))
        sg, sh = g.stats(k), h.stats(k)
        assert sg["total_iterations"] == sh["total_iterations"]
        assert sg["total_refinements"] == sh["total_refinements"]
    g.close()
    h.close()


@pytest.mark.parametrize("prec", [0, 2])
def test_autotune_restores_state(capi, oracle, prec):
    """The autotuner runs steps under every launch shape and puts the state back: after it the
    batch is at step 0 with its initial f, and the tuned launch shape solves to the same accuracy
    as the oracle (reduction order changes with the chunk size, so not bit for bit)."""
    probs = cases.batch_problems(6, seed=31, dt=1e-2, lo=20, hi=120)
    b = capi.Batch(probs, precision=prec)
    f0 = [b.f(k).copy() for k in range(len(probs))]
    chunk, grid = b.autotune(2)
    assert chunk in (1024, 2048, 4096) and grid in (8, 16, 32, 64)
    log = b.tuning_log()
    assert len(log) == 12 and all(e["ms_per_step"] > 0 for e in log)
    assert min(log, key=lambda e: e["ms_per_step"])["chunk"] == chunk
    for k in range(len(probs)):
        assert np.array_equal(b.f(k), f0[k])
        assert b.stats(k)["steps"] == 0
    b.step(3)
    tol = TOL64 if prec == 0 else TOL32
    for k, p in enumerate(probs):
        f = oracle.step(p, None, 3)
        assert rel(b.f(k), f) <= tol, (prec, k, rel(b.f(k), f))
        assert b.f(k).min() >= 0.0
    b.close()


def test_launch_shape_setter(capi):
    """Every launch shape gives the same FP64 answer up to the order of the reductions; shapes
    outside the supported set are refused."""
    probs = cases.batch_problems(4, seed=41, dt=1e-2, lo=30, hi=140)
    ref = capi.Batch(probs, precision=capi.FP64)
    ref.step(2)
    for chunk, blocks in ((1024, 8), (2048, 16), (4096, 32), (4096, 1)):
        b = capi.Batch(probs, precision=capi.FP64)
        b.set_launch_shape(chunk, blocks)
        assert b.launch_shape() == (chunk, blocks)
        b.step(2)
        for k in range(len(probs)):
            assert rel(b.f(k), ref.f(k)) <= 1e-12, (chunk, blocks, k)
        b.close()
    with pytest.raises(RuntimeError, match="chunk must be"):
        ref.set_launch_shape(3000, 8)
    with pytest.raises(RuntimeError, match="blocks_per_sm"):
        ref.set_launch_shape(1024, 0)
    ref.close()


@pytest.mark.parametrize("n,chunk", [(256, 1024), (512, 1024), (1024, 2048), (2048, 4096)])
def test_default_launch_shape(capi, n, chunk):
    """Without tuning, a batch takes the largest chunk that leaves at least two chunks per SM
    (GB300: 152 SMs, so 304 chunks): 512^2 cells make 128 chunks of 2048, 1024^2 make 256 of 4096
    but 512 of 2048, 2048^2 make 1024 of 4096."""
    s = capi.Solver(cases.synthetic_problem(n, n, 1e-2, seed=1), precision=capi.FP32_REFINE_DW)
    assert s.launch_shape()[0] == chunk
    s.close()


@pytest.mark.parametrize("pinned", [False, True])
@pytest.mark.parametrize("prec", [0, 2])
def test_step_host_round_trips_keep_history(capi, prec, pinned):
    """Stepping through host buffers that carry each step's output back in gives bit for bit the
    device-resident trajectory (the extrapolation history is kept); an instance whose state was
    changed on the host restarts its history, exactly as set_f on that instance does. Both
    pageable and page-locked (sayram_host_alloc) host buffers."""
    import ctypes

    probs = cases.batch_problems(4, seed=21, dt=1e-2, lo=30, hi=90)
    a = capi.Batch(probs, precision=prec)
    b = capi.Batch(probs, precision=prec)
    f0 = np.concatenate([p.f0.ravel() for p in probs])
    L = capi.load()
    if pinned:
        hp = [L.sayram_host_alloc(8 * f0.size) for _ in range(2)]
        fin, fout = [np.ctypeslib.as_array((ctypes.c_double * f0.size).from_address(h)) for h in hp]
        fin[:] = f0
    else:
        fin, fout = f0.copy(), np.empty_like(f0)
    a.step_host(1, fin.ctypes.data, fout.ctypes.data)
    b.step(1)
    for _ in range(4):
        fin[:] = fout
        a.step_host(1, fin.ctypes.data, fout.ctypes.data)
        b.step(1)
    for k in range(len(probs)):
        assert np.array_equal(a.f(k), b.f(k)), k
    off = probs[0].nx * probs[0].ny
    n1 = probs[1].nx * probs[1].ny
    fin[:] = fout
    fin[off:off + n1] *= 1.0 + 1e-9
    a.step_host(1, fin.ctypes.data, fout.ctypes.data)
    b.set_f(1, fin[off:off + n1].reshape(probs[1].nx, probs[1].ny))
    b.step(1)
    for k in range(len(probs)):
        assert np.array_equal(a.f(k), b.f(k)), k
    a.close()
    b.close()
    if pinned:
        for h in hp:
            L.sayram_host_free(h)


@pytest.mark.parametrize("prec", [0, 1, 2])
def test_stiff_steps(capi, oracle, prec):
    """Stiff settings: dt = 1 day (100 times the benchmark's), loss time 0.01 to 100 days, cross
    terms at |rho| = 0.99; six steps, so the extrapolated start runs at every order and through
    fast loss. Each mode still meets its tolerance against the oracle, stays non-negative and
    conserves mass."""
    probs = [cases.synthetic_problem(40 + 7 * k, 36 + 5 * k, 1.0, seed=90 + k, tau=tau, rho=rho)
             for k, (tau, rho) in enumerate(((0.01, 0.99), (100.0, -0.99), (0.3, 0.5), (None, -0.9)))]
    b = capi.Batch(probs, precision=prec)
    b.step(6)
    tol = TOL64 if prec == 0 else TOL32
    for k, p in enumerate(probs):
        ref = oracle.step(p, None, 6)
        f = b.f(k)
        st = b.stats(k)
        assert rel(f, ref) <= tol, (prec, k, rel(f, ref))
        assert f.min() >= 0.0 and st["status"] == 0 and st["mass_drift"] <= 1e-8, (prec, k, st)
    b.close()


@pytest.mark.parametrize("precond", [0, 1])
@pytest.mark.parametrize("prec", [0, 1, 2])
def test_preconditioners_meet_parity(capi, oracle, prec, precond):
    """Both inner-solve preconditioners (Jacobi scaling only; alpha-line 4-cell blocks, the
    default) give the reference's answer to each mode's tolerance on the small fixtures (ragged,
    1-wide, non-uniform, all-Dirichlet, all-zero-flux) and on stiff steps (dt = 1 day, |rho| =
    0.99, fast and no loss): the preconditioner steers the iteration, not the converged answer."""
    tol = TOL64 if prec == 0 else TOL32
    for name in NAMES:
        p = problem_from(Z, name)
        s = capi.Solver(p, precision=prec, precond=precond)
        s.step(10)
        f = s.f()
        st = s.get_stats()
        s.close()
        assert rel(f, Z[f"{name}/f10"]) <= tol, (name, prec, precond, rel(f, Z[f"{name}/f10"]))
        assert f.min() >= 0.0 and st["status"] == 0
    probs = [cases.synthetic_problem(40 + 7 * k, 36 + 5 * k, 1.0, seed=90 + k, tau=tau, rho=rho)
             for k, (tau, rho) in enumerate(((0.01, 0.99), (100.0, -0.99), (0.3, 0.5), (None, -0.9)))]
    b = capi.Batch(probs, precision=prec, precond=precond)
    b.step(4)
    for k, p in enumerate(probs):
        ref = oracle.step(p, None, 4)
        assert rel(b.f(k), ref) <= tol, (prec, precond, k, rel(b.f(k), ref))
        assert b.f(k).min() >= 0.0 and b.stats(k)["status"] == 0
    b.close()


@pytest.mark.parametrize("prec", [0, 2])
def test_alpha_line_blocks_cut_iterations(capi, prec):
    """On a stiff 256 x 256 instance (dt = 1e-2 day, the configuration of the single large
    instance) the alpha-line blocks take fewer inner iterations than Jacobi scaling alone, and both
    end at the same state to the mode's tolerance."""
    p = cases.synthetic_problem(256, 256, 1e-2, seed=11)
    out = {}
    for precond in (0, 1):
        s = capi.Solver(p, precision=prec, precond=precond)
        s.step(5)
        out[precond] = (s.f(), s.get_stats()["total_iterations"])
        s.close()
    tol = TOL64 if prec == 0 else TOL32
    assert rel(out[1][0], out[0][0]) <= tol
    assert out[1][1] < 0.8 * out[0][1], (prec, out[0][1], out[1][1])


def test_unknown_preconditioner_is_refused(capi):
    p = cases.synthetic_problem(8, 8, 1e-2, seed=1)
    with pytest.raises(RuntimeError, match="unknown preconditioner"):
        capi.Solver(p, precision=capi.FP64, precond=7)


def test_per_kernel_timing_of_the_cooperative_solve(capi):
    """With the cooperative solve, per-kernel timing names it beside the assembly and the polish,
    and the result is the same as stepping without timing."""
    probs = [cases.synthetic_problem(40 + 9 * k, 30 + 7 * k, 1e-2, seed=60 + k, tau=0.2 + k) for k in range(4)]
    a = capi.Batch(probs, precision=capi.FP32_REFINE_DW)
    b = capi.Batch(probs, precision=capi.FP32_REFINE_DW)
    a.enable_timing(True)
    a.step(2)
    kt = a.kernel_times()
    a.enable_timing(False)
    b.step(2)
    for k in range(len(probs)):
        assert np.array_equal(a.f(k), b.f(k))
    a.close()
    b.close()
    for name in ("begin", "assemble", "solve_coop", "polish"):
        assert name in kt and kt[name][1] == 2, (name, kt)
    assert "bicg1" not in kt and "resid" not in kt, kt


def test_per_kernel_timing_and_krylov_split(capi):
    """Per-kernel timing (host-loop steps bracketed by CUDA events) names every step kernel, and
    its split of the Krylov time -- whole BiCGSTAB iterations with fewer than / at least 10 % of
    the instances still iterating -- adds up to the three Krylov kernels' own time; the result is
    the same as stepping without timing."""
    probs = [cases.synthetic_problem(40 + 9 * k, 30 + 7 * k, 1e-2, seed=60 + k, tau=0.2 + k) for k in range(12)]
    a = capi.Batch(probs, precision=capi.FP32_REFINE_DW)
    b = capi.Batch(probs, precision=capi.FP32_REFINE_DW)
    a.set_coop(False)  # a batch this small would run its loop as one cooperative kernel
    a.enable_timing(True)
    a.step(3)
    kt = a.kernel_times()
    a.enable_timing(False)
    b.step(3)
    for k in range(len(probs)):
        assert np.array_equal(a.f(k), b.f(k))
    a.close()
    b.close()
    for name in ("begin", "assemble", "resid", "bicg1", "bicg2", "bicg3", "polish", "krylov_rest"):
        assert name in kt and kt[name][1] > 0, (name, kt)
    kry = sum(kt[n][0] for n in ("bicg1", "bicg2", "bicg3"))
    split = kt["krylov_rest"][0] + kt.get("krylov_tail10", (0.0, 0))[0]
    assert kry <= split * 1.001 and split <= kry * 1.5 + 0.5, (kry, split)
    n_iter = kt["krylov_rest"][1] + kt.get("krylov_tail10", (0.0, 0))[1]
    assert n_iter == kt["bicg1"][1] == kt["bicg3"][1]
