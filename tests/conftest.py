import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import __graft_entry__  # noqa: E402

__graft_entry__.load_package()

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built CUDA library")
    config.addinivalue_line("markers", "slow: long-running")


@pytest.fixture(scope="session")
def oracle():
    import oracle as orc  # the checker (tests only)

    orc.build()
    return orc


@pytest.fixture(scope="session")
def capi():
    """The CUDA library binding; GPU tests fail loudly if it cannot be loaded."""
    from sayram2d_gb300 import build, capi as c

    build.build()
    c.load()
    return c


def load_small():
    """The reference-generated fixtures of the small cases: (npz, case names)."""
    import numpy as np

    z = np.load(os.path.join(GOLDEN, "ref_small.npz"))
    names = sorted({k.split("/")[0] for k in z.files})
    return z, names


def problem_from(z, name):
    """Rebuilds a cases.Problem from its stored inputs."""
    from sayram2d_gb300 import cases

    g = lambda k: z[f"{name}/{k}"]
    meta = g("meta")
    nx, ny, dt = int(meta[0]), int(meta[1]), float(meta[2])
    bc = [int(v) for v in meta[3:7]]
    dirs = [g(f"dir{s}") if bc[s] == cases.DIRICHLET else None for s in range(4)]
    return cases.Problem(nx, ny, g("x_edges"), g("y_edges"), dt, bc, g("G"), g("Dxx"), g("Dxy"),
                         g("Dyy"), g("inv_tau"), g("f0"), dirs, name=name)


def c0_problem():
    from sayram2d_gb300 import cases

    rp = cases.read_ini(os.path.join(ROOT, "sayram-2d_gb300", "configs", "c0.ini"))
    return rp, cases.problem_from_params(rp)


def load_table_cases():
    """The reference-generated Albert_Young / Albert_Young_LC fixtures: name -> dict with which,
    x_edges, y_edges, dt, Emin, Emax, table (cases.DTable) and the reference's outputs (G, Dxx,
    Dxy, Dyy, inv_tau, f0, bc, dirichlet)."""
    import numpy as np
    from sayram2d_gb300 import cases

    z = np.load(os.path.join(GOLDEN, "ref_cases.npz"))
    out = {}
    for name in sorted({k.split("/")[0] for k in z.files}):
        g = lambda k: z[f"{name}/{k}"]
        which, dt, Emin, Emax = g("meta")
        bc = [int(v) for v in g("bc")]
        out[name] = {
            "which": int(which), "dt": float(dt), "Emin": float(Emin), "Emax": float(Emax),
            "x_edges": g("x_edges"), "y_edges": g("y_edges"),
            "table": cases.DTable(*[g("table_" + k) for k in ("alpha0_deg", "E", "Daa", "Dap", "Dpp")]),
            **{k: g(k) for k in ("G", "Dxx", "Dxy", "Dyy", "inv_tau", "f0")},
            "bc": bc, "dirichlet": [g(f"dir{s}") if bc[s] == cases.DIRICHLET else None for s in range(4)],
        }
    return out


def ay80_table():
    """The reference's D table (D/AlbertYoung_chorus.h5) as stored in the fixture."""
    import numpy as np
    from sayram2d_gb300 import cases

    z = np.load(os.path.join(GOLDEN, "ref_ay_80x80.npz"))
    return cases.DTable(*[z["table_" + k] for k in ("alpha0_deg", "E", "Daa", "Dap", "Dpp")])


def ay80_problem(name="ay"):
    """The reference's own run configurations fed its own D table: ``ay`` (p.ini: Albert_Young,
    80 x 80, alpha0 from 5 deg, dt = 2e-3) or ``lc`` (p_AlbertYoungLC.ini: Albert_Young_LC, alpha0
    from 0 deg). Returns (problem with the fields the reference's case built, {steps: f of the
    reference's Solver after that many steps}); saves every 50 steps up to 500."""
    import numpy as np
    from sayram2d_gb300 import cases

    z = np.load(os.path.join(GOLDEN, "ref_ay_80x80.npz"))
    g = lambda k: z[f"{name}/{k}"]
    which, dt, Emin, Emax = g("meta")
    bc = [int(v) for v in g("bc")]
    dirs = [g(f"dir{s}") if bc[s] == cases.DIRICHLET else None for s in range(4)]
    p = cases.Problem(80, 80, g("x_edges"), g("y_edges"), float(dt), bc, g("G"), g("Dxx"), g("Dxy"),
                      g("Dyy"), g("inv_tau"), g("f0"), dirs, name=f"ay80_{name}")
    return p, {int(n): g(f"f{int(n)}") for n in z["saves"]}


def reference_tree():
    """The reference's source tree when this machine has it (oracle.reference_root), else None."""
    import oracle as orc  # the checker (tests only)

    return orc.reference_root()


def case_problem(c):
    """A cases.Problem for a table fixture, built by the host case generators with the
    reference's interpolated D (the generators' G, f0 and inv_tau are compared separately)."""
    from sayram2d_gb300 import cases

    nx, ny = len(c["x_edges"]) - 1, len(c["y_edges"]) - 1
    mk = cases.albert_young_problem if c["which"] == 0 else cases.albert_young_lc_problem
    kw = {"alpha0_min_deg": 5.0} if c["which"] == 0 else {}
    return mk(nx, ny, c["dt"], Emin=c["Emin"], Emax=c["Emax"], D=(c["Dxx"], c["Dxy"], c["Dyy"]), **kw)
