"""Serving (continuous batching): requests of different grid sizes and step counts arrive while
others run; each result must equal the same request run alone (FP64: 1e-12, FP32 modes: 1e-8 in
relative L2), admission respects the HBM budget, and oversized requests are refused."""
import ctypes

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


def test_tick_gives_up_after_its_wait_limit_and_a_later_tick_collects(capi):
    """The host wait of a tick is bounded (sayram_server_config.wait_seconds): with a limit of a
    microsecond, a legitimately long step (a 512 x 512 FP64 request) is still running when the
    tick gives up and returns SAYRAM_ERR_TIMEOUT; the step stays in flight, later ticks wait for it
    again, and the result is the request alone. Nothing on the GPU waits or hangs: only the host
    stops waiting."""
    p = cases.synthetic_problem(512, 512, 1e-2, seed=7)
    srv = capi.Server(4e9, max_slots=4, max_side=512, precision=capi.FP64, wait_seconds=1e-6)
    rid = srv.submit(p, 3)
    L = capi.load()
    n = ctypes.c_int(0)
    rc = L.sayram_server_tick(srv.h, ctypes.byref(n))
    assert rc == capi.ERR_TIMEOUT, (rc, capi.last_error())
    assert "still running" in capi.last_error()
    got = None
    for _ in range(100000):
        rc = L.sayram_server_tick(srv.h, ctypes.byref(n))
        assert rc in (capi.OK, capi.ERR_TIMEOUT), capi.last_error()
        got = srv.poll(rid)
        if got is not None:
            break
    info = srv.info()
    srv.close()
    assert got is not None and info["completed"] == 1
    f, st, _, _ = got
    assert st["steps"] == 3
    ref = _alone(capi, p, 3, capi.FP64)
    assert rel(f, ref) <= 1e-12
