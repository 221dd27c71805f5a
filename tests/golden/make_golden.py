"""Generates the golden fixtures in this directory from the reference's OWN solver sources.

Sayram-2D's source/Solver.cc and source/Mesh.cc are compiled unmodified against the project's
Eigen/xtensor shim headers (``make -C oracle ref`` -> oracle/_ref/libsayram_ref.so) and driven by
oracle/ref_harness.cc. For every case this script stores the inputs, the matrix M (five
diagonals, system order) and right-hand side R that the reference assembles from f0, and f after
1 and ``nsteps`` updates. The config-0 case (90 x 90, 1000 steps) stores only outputs; its inputs
are regenerated from the seeded generator (an input checksum guards against drift).

The case fixtures (ref_cases.npz) come from the reference's own Albert_Young, Albert_Young_LC
and Albert_Young_IO sources, compiled the same way (oracle/_ref/libsayram_case_ref.so, driven by
oracle/ref_case_harness.cc): for each grid and seeded D table, the fields a Solver reads from the
case -- G, Dxx, Dxy, Dyy (interpolated from the table), inv_tau, init_f, the BC types and the
Dirichlet vertex values.

The config-1 prefix (ref_c1_1024_prefix.npz: one 1024 x 1024 instance, dt = 1e-2, f after 1 and
10 steps) is too large for the reference's build here, whose LU shim is a banded elimination
(bandwidth 1024). It comes from the C restatement of the reference's assembly (bit-exact with the
reference build on every small fixture) and SciPy's SuperLU with COLAMD, the algorithm family
of the reference's Eigen SparseLU; it stores a strided sample of f (every 8th cell in each
direction), the row and column sums of f and its sum of squares, plus an input digest.

ref_ay_80x80.npz is the reference's own run configurations (p.ini: Albert_Young, 80 x 80, alpha0
from 5 deg, 500 steps of dt = 2e-3, saved every 50 steps; p_AlbertYoungLC.ini: the same with
alpha0 from 0 deg, run with Albert_Young_LC) fed the reference's own D table,
D/AlbertYoung_chorus.h5, read by the library's HDF5 reader (sayram_dtable_load_h5): the table's
values (so that tests can write the D file anywhere, the GPU host included), the case fields from
the reference's Albert_Young / Albert_Young_LC, and f at every save (/f/1 .. /f/10) of the
reference's own Solver.

The reference tree is $SAYRAM_REFERENCE (default /root/reference). Run where it exists:
  python tests/golden/make_golden.py [cases|ay80|config1|config1_full]
("cases" regenerates only ref_cases.npz, "ay80" the case fixtures and ref_ay_80x80.npz,
"config1" only the config-1 prefix, ~6 min, "config1_full" the 500-step config-1 fixture
ref_c1_1024_full.npz, about an hour on one core)

ref_c1_1024_full.npz pins config 1 over all 500 steps with the tight-residual solve
(oracle.solve_tight), which agrees with the SuperLU prefix to <= 1e-12 over its 10 steps.
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import __graft_entry__  # noqa: E402

__graft_entry__.load_package()
from sayram2d_gb300 import cases  # noqa: E402

import oracle  # noqa: E402

PI = cases.PI


def small_cases():
    D, Z = cases.DIRICHLET, cases.ZEROFLUX
    out = {
        "syn_6x5": cases.synthetic_problem(6, 5, 1e-3, seed=3),
        "syn_7x7_dt1e-2": cases.synthetic_problem(7, 7, 1e-2, seed=4, tau=0.5),
        "ay_8x6": cases.albert_young_problem(8, 6, 1e-2),
        "lc_9x4": cases.albert_young_lc_problem(9, 4, 1e-2),
        "syn_1x5": cases.synthetic_problem(1, 5, 1e-2, seed=5),
        "syn_5x1": cases.synthetic_problem(5, 1, 1e-2, seed=6),
        "syn_1x1": cases.synthetic_problem(1, 1, 1e-2, seed=7),
        "syn_17x13_nonuniform": cases.synthetic_problem(
            17, 13, 1e-2, seed=8, x_edges=cases.stretched_edges(17, 5 * PI / 180, PI / 2, 0.6),
            y_edges=cases.stretched_edges(13, np.log(0.2), np.log(5.0), -0.5)),
        "syn_33x20_zeroflux": cases.synthetic_problem(33, 20, 1e-2, seed=9, bc=[Z, Z, Z, Z]),
        "syn_20x33_alldirichlet": cases.synthetic_problem(20, 33, 1e-2, seed=10, bc=[D, D, D, D]),
        "syn_24x18_rho-0.9": cases.synthetic_problem(24, 18, 1e-2, seed=11, rho=-0.9, tau=0.1),
        "syn_24x18_rho+0.9_notau": cases.synthetic_problem(24, 18, 1e-2, seed=12, rho=0.9, tau=None),
    }
    return out


def pack_problem(p, prefix):
    d = {}
    for k in ("x_edges", "y_edges", "G", "Dxx", "Dxy", "Dyy", "inv_tau", "f0"):
        d[prefix + k] = getattr(p, k)
    d[prefix + "meta"] = np.array([p.nx, p.ny, p.dt, *p.bc], dtype=np.float64)
    for s in range(4):
        d[prefix + f"dir{s}"] = p.dirichlet[s] if p.dirichlet[s] is not None else np.zeros(0)
    return d


def input_digest(p):
    h = hashlib.sha256()
    for k in ("x_edges", "y_edges", "G", "Dxx", "Dxy", "Dyy", "inv_tau", "f0"):
        h.update(np.ascontiguousarray(getattr(p, k)).tobytes())
    return h.hexdigest()


def table_cases():
    """(which, x_edges, y_edges, dt, Emin, Emax, table) per fixture; which 0 = Albert_Young,
    1 = Albert_Young_LC. The grids follow main.cc:20-37; the tables are seeded stand-ins for the
    HDF5 D files, one of them ending below the grid's upper alpha0 and E (the clamped branch of
    calWeight), one of them the smallest table (2 x 2)."""
    d2r = PI / 180
    lE = lambda lo, hi, n: cases.uniform_edges(n, np.log(lo), np.log(hi))
    return {
        "ay_24x20": (0, cases.uniform_edges(24, 5 * d2r, 90 * d2r), lE(0.2, 5.0, 20), 1e-2, 0.2, 5.0,
                     cases.synthetic_dtable(1)),
        "ay_16x12_clamped": (0, cases.uniform_edges(16, 5 * d2r, 90 * d2r), lE(0.2, 5.0, 12), 1e-2, 0.2, 5.0,
                             cases.synthetic_dtable(2, n_alpha=31, n_E=17, alpha0_max_deg=60.0, Emax=2.0)),
        "lc_20x16": (1, cases.uniform_edges(20, 0.0, 90 * d2r), lE(0.2, 5.0, 16), 1e-2, 0.2, 5.0,
                     cases.synthetic_dtable(3)),
        "ay_13x9_table2x2": (0, cases.uniform_edges(13, 5 * d2r, 90 * d2r), lE(0.2, 5.0, 9), 1e-3, 0.2, 5.0,
                             cases.synthetic_dtable(4, n_alpha=2, n_E=2)),
    }


def write_case_fixtures():
    data = {}
    for name, (which, xe, ye, dt, Emin, Emax, t) in table_cases().items():
        r = oracle.ref_case(which, xe, ye, dt, Emin, Emax, t)
        data[name + "/meta"] = np.array([which, dt, Emin, Emax], dtype=np.float64)
        data[name + "/x_edges"], data[name + "/y_edges"] = xe, ye
        for k in ("alpha0_deg", "E", "Daa", "Dap", "Dpp"):
            data[name + "/table_" + k] = getattr(t, k)
        for k in ("G", "Dxx", "Dxy", "Dyy", "inv_tau", "f0"):
            data[name + "/" + k] = r[k]
        data[name + "/bc"] = np.array(r["bc"], dtype=np.float64)
        for s in range(4):
            data[name + f"/dir{s}"] = r["dirichlet"][s] if r["dirichlet"][s] is not None else np.zeros(0)
    np.savez_compressed(os.path.join(HERE, "ref_cases.npz"), **data)


REFERENCE = os.environ.get("SAYRAM_REFERENCE") or "/root/reference"
AY80_SAVES = tuple(range(50, 501, 50))


def ay80_table():
    """The reference's D table D/AlbertYoung_chorus.h5 (p.ini:25-26), read by the library's HDF5
    reader."""
    from sayram2d_gb300 import build, capi

    build.build()
    return capi.load_dtable(os.path.join(REFERENCE, "D", "AlbertYoung_chorus.h5"))


def ay80_cases():
    """p.ini:1-27 and p_AlbertYoungLC.ini: 80 x 80 cells, E from 0.2 to 5 MeV, T = 1 day in 500
    steps (dt = 2e-3); alpha0 from 5 deg (Albert_Young, which 0) or 0 deg (Albert_Young_LC,
    which 1) to 90 deg (main.cc:20-37)."""
    d2r = PI / 180
    ye = cases.uniform_edges(80, np.log(0.2), np.log(5.0))
    return {"ay": (0, cases.uniform_edges(80, 5 * d2r, 90 * d2r), ye),
            "lc": (1, cases.uniform_edges(80, 0 * d2r, 90 * d2r), ye)}


def write_ay80():
    t = ay80_table()
    dt, Emin, Emax = 1.0 / 500, 0.2, 5.0
    data = {"saves": np.array(AY80_SAVES)}
    for k in ("alpha0_deg", "E", "Daa", "Dap", "Dpp"):
        data["table_" + k] = getattr(t, k)
    for name, (which, xe, ye) in ay80_cases().items():
        r = oracle.ref_case(which, xe, ye, dt, Emin, Emax, t)
        data[name + "/meta"] = np.array([which, dt, Emin, Emax], dtype=np.float64)
        data[name + "/x_edges"], data[name + "/y_edges"] = xe, ye
        for k in ("G", "Dxx", "Dxy", "Dyy", "inv_tau", "f0"):
            data[name + "/" + k] = r[k]
        data[name + "/bc"] = np.array(r["bc"], dtype=np.float64)
        for s in range(4):
            data[name + f"/dir{s}"] = r["dirichlet"][s] if r["dirichlet"][s] is not None else np.zeros(0)
        p = cases.Problem(80, 80, xe, ye, dt, list(r["bc"]), r["G"], r["Dxx"], r["Dxy"], r["Dyy"],
                          r["inv_tau"], r["f0"], list(r["dirichlet"]), name="ay80_" + name)
        for n in AY80_SAVES:
            _, _, f = oracle.ref_run(p, n)
            data[name + f"/f{n}"] = f
    np.savez_compressed(os.path.join(HERE, "ref_ay_80x80.npz"), **data)


def config1_problem():
    return cases.synthetic_problem(1024, 1024, 1e-2, seed=11)


def write_config1_prefix(nsteps=10):
    p = config1_problem()
    out = {"digest": np.frombuffer(bytes.fromhex(input_digest(p)), dtype=np.uint8),
           "nsteps": np.array([nsteps])}
    f = oracle.step(p, None, 1, solver="splu")
    out["f1_sub"] = f[::8, ::8].copy()
    out["f1_rows"], out["f1_cols"] = f.sum(axis=1), f.sum(axis=0)
    f = oracle.step(p, f, nsteps - 1, solver="splu")
    out["fN_sub"] = f[::8, ::8].copy()
    out["fN_rows"], out["fN_cols"] = f.sum(axis=1), f.sum(axis=0)
    out["fN_ssq"] = np.array([float((f * f).sum())])
    out["fN_min"] = np.array([float(f.min())])
    np.savez_compressed(os.path.join(HERE, "ref_c1_1024_prefix.npz"), **out)


C1_SAVES = (10, 100, 250, 500)


def write_config1_full(nsteps=500):
    """Config 1 over all 500 steps: the restated assembly and the tight-residual solve
    (oracle.solve_tight: BiCGSTAB with an alpha-line preconditioner inside iterative refinement,
    residuals in extended precision, down to the rounding floor of a float64 solution), warm
    started from the previous step. Stores, at steps 10, 100, 250 and 500, a strided sample of f,
    its row and column sums, sum of squares and minimum, plus the largest relative residual of
    any step; the first 10 steps are also checked against the SuperLU prefix fixture (the direct
    solve), and the agreement is stored."""
    import time

    p = config1_problem()
    z = np.load(os.path.join(HERE, "ref_c1_1024_prefix.npz"))
    out = {"digest": np.frombuffer(bytes.fromhex(input_digest(p)), dtype=np.uint8),
           "saves": np.array(C1_SAVES)}
    f = p.f0.copy()
    worst, iters, t0 = 0.0, 0, time.time()
    for k in range(1, nsteps + 1):
        M5, R = oracle.assemble(p, f)
        x, rel, its = oracle.solve_tight(p.nx, p.ny, M5, R, oracle.field_to_sys(f))
        f = oracle.sys_to_field(p.nx, p.ny, x)
        worst, iters = max(worst, rel), iters + its
        if k in (1, 10):
            pre = "f1" if k == 1 else "fN"
            agree = max(float(np.linalg.norm(f[::8, ::8] - z[pre + "_sub"]) / np.linalg.norm(z[pre + "_sub"])),
                        float(np.linalg.norm(f.sum(axis=1) - z[pre + "_rows"]) / np.linalg.norm(z[pre + "_rows"])))
            out[f"agree_superlu_step{k}"] = np.array([agree])
            print(f"step {k}: tight vs SuperLU {agree:.2e}", flush=True)
            assert agree <= 1e-12, agree
        if k in C1_SAVES:
            out[f"f{k}_sub"] = f[::8, ::8].copy()
            out[f"f{k}_rows"], out[f"f{k}_cols"] = f.sum(axis=1), f.sum(axis=0)
            out[f"f{k}_ssq"] = np.array([float((f * f).sum())])
            out[f"f{k}_min"] = np.array([float(f.min())])
        if k % 10 == 0:
            print(f"step {k}: rel {rel:.2e} its {its} ({time.time() - t0:.0f} s)", flush=True)
    out["max_rel_residual"] = np.array([worst])
    out["inner_iterations"] = np.array([iters])
    np.savez_compressed(os.path.join(HERE, "ref_c1_1024_full.npz"), **out)


def main():
    oracle.build()
    if sys.argv[1:] == ["config1"]:
        write_config1_prefix()
        print("wrote ref_c1_1024_prefix.npz")
        return
    if sys.argv[1:] == ["config1_full"]:
        write_config1_full()
        print("wrote ref_c1_1024_full.npz")
        return
    if oracle.build_ref(REFERENCE) is None:
        raise SystemExit("the reference sources are needed to generate fixtures ($SAYRAM_REFERENCE)")
    write_case_fixtures()
    if sys.argv[1:] == ["cases"]:
        print("wrote ref_cases.npz")
        return
    write_ay80()
    if sys.argv[1:] == ["ay80"]:
        print("wrote ref_ay_80x80.npz")
        return
    nsteps = 10
    data = {}
    for name, p in small_cases().items():
        M5, R, f1 = oracle.ref_run(p, 1)
        _, _, fN = oracle.ref_run(p, nsteps)
        data.update(pack_problem(p, name + "/"))
        data[name + "/M5"] = M5
        data[name + "/R"] = R
        data[name + "/f1"] = f1
        data[name + f"/f{nsteps}"] = fN
    np.savez_compressed(os.path.join(HERE, "ref_small.npz"), **data)
    # config 0: ini-driven 90 x 90, dt = 1e-3, 1000 steps
    rp = cases.read_ini(os.path.join(ROOT, "sayram-2d_gb300", "configs", "c0.ini"))
    p = cases.problem_from_params(rp)
    out = {"digest": np.frombuffer(bytes.fromhex(input_digest(p)), dtype=np.uint8)}
    for n in (1, 100, rp.nsteps):
        _, _, f = oracle.ref_run(p, n)
        out[f"f{n}"] = f
    np.savez_compressed(os.path.join(HERE, "ref_c0_90x90.npz"), **out)
    print("wrote", sorted(os.listdir(HERE)))


if __name__ == "__main__":
    main()
