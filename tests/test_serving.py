"""Serving (continuous batching): requests of different grid sizes and step counts arrive while
others run; each result must equal the same request run alone (FP64: 1e-12, FP32 modes: 1e-8 in
relative L2), admission respects the HBM budget, and oversized requests are refused."""
import numpy as np
import pytest

from sayram2d_gb300 import cases

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _alone(capi, p, nsteps, prec):
    s = capi.Solver(p, precision=prec)
    s.step(nsteps)
    f = s.f()
    s.close()
    return f


def _requests():
    shapes = [(40, 33, 7), (96, 80, 12), (33, 64, 3), (128, 120, 9), (64, 64, 15), (17, 23, 5)]
    return [(cases.synthetic_problem(a, e, 1e-2, seed=100 + k, tau=0.3 + 0.2 * k), n)
            for k, (a, e, n) in enumerate(shapes)]


@pytest.mark.parametrize("lanes", [1, 2])
@pytest.mark.parametrize("prec,tol", [(0, 1e-12), (2, 1e-8), (1, 1e-8)])
def test_same_alone_and_in_the_mix(capi, prec, tol, lanes):
    """With two lanes (max side <= 64 in the first), the four small requests and the two large
    ones step in separate lanes at their own pace; every result is still the request alone."""
    reqs = _requests()
    srv = capi.Server(2e9, max_slots=16, max_side=256, precision=prec, lanes=lanes, split_side=64)
    ids = {}
    # staggered arrivals: two at once, then one per tick while the others run
    ids[srv.submit(*reqs[0])] = 0
    ids[srv.submit(*reqs[1])] = 1
    pending = list(range(2, len(reqs)))
    got = {}
    for _ in range(200):
        if pending:
            k = pending.pop(0)
            ids[srv.submit(*reqs[k])] = k
        srv.tick()
        for rid in list(ids):
            r = srv.poll(rid)
            if r is not None:
                got[ids.pop(rid)] = r
        if not ids and not pending:
            break
    info = srv.info()
    srv.close()
    assert len(got) == len(reqs) and info["completed"] == len(reqs) and info["submitted"] == len(reqs)
    assert info["resident"] == 0 and info["waiting"] == 0
    for k, (p, n) in enumerate(reqs):
        f, st, t0, t1 = got[k]
        assert st["steps"] == n and t1 >= t0
        assert f.min() >= 0.0 and st["min_f"] >= 0.0
        assert rel(f, _alone(capi, p, n, prec)) <= tol, (prec, k)


def test_admission_waits_for_memory(capi):
    """An arena that holds one instance but not two: later requests wait, then run, all correct."""
    region = lambda n: ((n + 2) * ((n + 3) // 4 * 4) + 31) // 32 * 32
    n = 64
    budget = None
    for b in np.arange(68e6, 90e6, 0.25e6):  # find a budget whose arena fits one 64x64, not two
        try:
            probe = capi.Server(float(b), max_slots=8, max_side=128, precision=capi.FP32_REFINE_DW)
        except RuntimeError:  # below the server's fixed reserve
            continue
        arena = probe.info()["arena_cells"]
        probe.close()
        if region(n) <= arena < 2 * region(n):
            budget = float(b)
            break
    assert budget is not None
    reqs = [(cases.synthetic_problem(n, n, 1e-2, seed=200 + k), 3 + k) for k in range(3)]
    srv = capi.Server(budget, max_slots=8, max_side=128, precision=capi.FP32_REFINE_DW)
    ids = {srv.submit(p, m): k for k, (p, m) in enumerate(reqs)}
    srv.tick()
    info = srv.info()
    assert info["resident"] == 1 and info["waiting"] == 2
    got = {}
    for _ in range(200):
        srv.tick()
        for rid in list(ids):
            r = srv.poll(rid)
            if r is not None:
                got[ids.pop(rid)] = r
        if not ids:
            break
    srv.close()
    assert len(got) == 3
    for k, (p, m) in enumerate(reqs):
        assert rel(got[k][0], _alone(capi, p, m, capi.FP32_REFINE_DW)) <= 1e-8


def test_lane_configuration_checked(capi):
    with pytest.raises(RuntimeError, match="lane_split_side"):
        capi.Server(1e9, max_slots=4, max_side=128, precision=capi.FP32_REFINE_DW, lanes=2, split_side=128)
    srv = capi.Server(1e9, max_slots=4, max_side=128, precision=capi.FP32_REFINE_DW, lanes=2, split_side=32)
    with pytest.raises(RuntimeError, match="max_side"):
        srv.submit(cases.synthetic_problem(130, 20, 1e-2, seed=1), 2)
    srv.close()


def test_oversized_request_refused(capi):
    srv = capi.Server(600e6, max_slots=4, max_side=64, precision=capi.FP32_REFINE_DW)
    p = cases.synthetic_problem(100, 50, 1e-2, seed=1)
    with pytest.raises(RuntimeError, match="max_side"):
        srv.submit(p, 3)
    srv.close()
