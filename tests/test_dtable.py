"""GPU: D fields interpolated on the device from a D table (sayram_set_dtable /
sayram_batch_set_dtable) against the oracle's restatement of the Albert_Young cases' constructD,
which is bit-exact against the reference's own case code (tests/test_oracle.py). The host-side
row factors (exp, log, pow) come from the same libm as the oracle's, and every device operation
is a separately rounded IEEE add, multiply or divide in the reference's order, so the assembled
systems are compared bit for bit."""
import numpy as np
import pytest

from conftest import case_problem, load_table_cases
from sayram2d_gb300 import cases

pytestmark = pytest.mark.gpu

TABLE_CASES = load_table_cases()


def _reference_table_cases():
    """The reference's own D table (D/AlbertYoung_chorus.h5) on the grids of its run files, with
    the fields the reference's Albert_Young / Albert_Young_LC built from it."""
    from conftest import ay80_problem, ay80_table

    out = {}
    for name, which in (("ay", 0), ("lc", 1)):
        p, _ = ay80_problem(name)
        out["ref_table_" + name + "_80x80"] = {
            "which": which, "dt": p.dt, "Emin": 0.2, "Emax": 5.0, "x_edges": p.x_edges, "y_edges": p.y_edges,
            "table": ay80_table(), "G": p.G, "Dxx": p.Dxx, "Dxy": p.Dxy, "Dyy": p.Dyy, "inv_tau": p.inv_tau,
            "f0": p.f0, "bc": p.bc, "dirichlet": p.dirichlet}
    return out


TABLE_CASES.update(_reference_table_cases())


def with_D(p, D):
    q = cases.Problem(p.nx, p.ny, p.x_edges, p.y_edges, p.dt, list(p.bc), p.G, *D, p.inv_tau, p.f0,
                      p.dirichlet, name=p.name)
    return q


def test_oracle_tables_agree_across_machines(oracle):
    """The oracle on this machine reproduces the reference fixture to a few ulps (libm may differ
    between the machine that made the fixture and this one)."""
    for name, c in TABLE_CASES.items():
        D = oracle.dtable_fields(c["x_edges"], c["y_edges"], c["table"])
        for k, d in zip(("Dxx", "Dxy", "Dyy"), D):
            assert np.allclose(d, c[k], rtol=1e-14, atol=0.0), (name, k)


@pytest.mark.parametrize("prec", [0, 2])
@pytest.mark.parametrize("name", sorted(TABLE_CASES))
def test_set_dtable_equals_host_fields(capi, oracle, name, prec):
    c = TABLE_CASES[name]
    base = case_problem(c)
    D = oracle.dtable_fields(c["x_edges"], c["y_edges"], c["table"])
    a = capi.Solver(with_D(base, D), precision=prec)
    # start from other D fields, then replace them from the table on the device
    b = capi.Solver(with_D(base, (2.0 * D[0], 0.5 * D[1], 3.0 * D[2])), precision=prec)
    b.set_dtable(c["table"])
    Ma, Ra = a.export_system(0)
    Mb, Rb = b.export_system(0)
    assert np.array_equal(Ma, Mb) and np.array_equal(Ra, Rb), (name, prec, np.abs(Ma - Mb).max())
    a.step(3)
    b.step(3)
    assert np.array_equal(a.f(), b.f())
    if prec == 0:
        ref = oracle.step(with_D(base, D), None, 3)
        assert np.linalg.norm(b.f() - ref) <= 1e-10 * np.linalg.norm(ref)
    a.close()
    b.close()


def test_batch_set_dtable_all_instances(capi, oracle):
    """idx < 0: one launch interpolates the same table onto every instance's own grid."""
    t = TABLE_CASES["ay_24x20"]["table"]
    probs, Ds = [], []
    for c in TABLE_CASES.values():
        base = case_problem(c)
        D = oracle.dtable_fields(c["x_edges"], c["y_edges"], t)
        probs.append(with_D(base, (D[0] * 1.5, D[1], D[2] * 0.25)))
        Ds.append(D)
    b = capi.Batch(probs, precision=capi.FP64)
    b.set_dtable(-1, t)
    for k, (p, D) in enumerate(zip(probs, Ds)):
        s = capi.Solver(with_D(p, D), precision=capi.FP64)
        M1, R1 = s.export_system(0)
        M2, R2 = b.export_system(k)
        assert np.array_equal(M1, M2) and np.array_equal(R1, R2), k
        s.close()
    b.close()


def test_set_dtable_rejects_bad_tables(capi):
    c = TABLE_CASES["ay_24x20"]
    s = capi.Solver(case_problem(c), precision=capi.FP64)
    t = c["table"]
    bad = cases.DTable(t.alpha0_deg[:1], t.E, t.Daa[:1], t.Dap[:1], t.Dpp[:1])
    with pytest.raises(RuntimeError, match="n_alpha, n_energy >= 2"):
        s.set_dtable(bad)
    rev = cases.DTable(t.alpha0_deg[::-1].copy(), t.E, t.Daa, t.Dap, t.Dpp)
    with pytest.raises(RuntimeError, match="must increase"):
        s.set_dtable(rev)
    with pytest.raises(RuntimeError, match="out of range"):
        capi.Batch.set_dtable(s, 5, t)
    s.close()
