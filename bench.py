#!/usr/bin/env python3
"""Benchmark of the Sayram-2D hot path on one GB300.

Workload (the batched mixed-precision configuration the headline metric is quoted on): 4096
independent instances, nalpha and nE each uniform in [64, 256], seeded synthetic D fields
(rho ~ U[-0.9, 0.9], tau log-uniform in [0.1, 10] days), dt = 1e-2 day, advanced together with an
FP32 Krylov solve (alpha-line block preconditioner) inside double-word (FP32-pair) residual and
refinement, to a relative residual of 1e-11. One bench "step" is one backward-Euler step of every
instance (assembly, solve, positivity polish).

Prints ONE JSON line:
  value        instance-steps/s, device-timed (CUDA events on the batch stream), inputs resident
  e2e          the same metric through sayram_batch_step_host with pinned host buffers: every step
               copies all instances' f host->device and the result device->host
  roofline     the dominant kernel: the analysis' algorithmic bytes / event-timed duration vs the
               measured HBM copy bandwidth (the design's own byte model beside it)
  cpu_baseline the oracle port (C assembly restatement + SuperLU/COLAMD, the algorithm family of
               the reference's Eigen SparseLU) on one host core, on a bounded sample
  plain_fp64   the single-instance FP64 drop-in (sayram_create/sayram_update) on a sample of the
               same batch, one instance after another
and accuracy: rel L2 error against the oracle on a size-spread sample of the batch and against
the batched FP64 path, min cell, mass drift; the other arithmetic and preconditioner on the same
batch; the 1024^2 single instance; serving latency (Poisson stream) and serving capacity (a burst
against plain-FP64 serving and the one-at-a-time drop-in).

--impl reference times the oracle port on all host cores instead (the reference's own build needs
Eigen/xtensor/HDF5, which are not available here).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

import __graft_entry__  # noqa: E402

__graft_entry__.load_package()
from sayram2d_gb300 import cases  # noqa: E402

METRIC = "instance-steps/s batched FP32+refine vs plain FP64 (rel err<=1e-8); p50/p99 ms"
UNIT = "instance-steps/s"
DT = 1e-2


class Ranks:
    """One process per GPU under torchrun (RANK / LOCAL_RANK / WORLD_SIZE from the environment).
    Instances are independent, so each rank steps its own shard of the batch and nothing crosses
    between GPUs on the data path; the process group only lines the ranks up around the timed
    region and takes the maximum of their times (NCCL on GPUs, gloo without). A single process
    (no torchrun) needs no process group."""

    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", str(self.rank)))
        self.dist = None
        self.device = None
        if self.world > 1:
            import torch
            import torch.distributed as dist

            if torch.cuda.is_available():
                torch.cuda.set_device(self.local)
                self.device = torch.device("cuda", self.local)
                dist.init_process_group("nccl")
            else:
                self.device = torch.device("cpu")
                dist.init_process_group("gloo")
            self.dist = dist
            self._torch = torch

    def barrier(self) -> None:
        if self.dist is not None:
            self.dist.barrier()

    def _reduce(self, x: float, op) -> float:
        if self.dist is None:
            return float(x)
        t = self._torch.tensor([float(x)], dtype=self._torch.float64, device=self.device)
        self.dist.all_reduce(t, op=op)
        return float(t.item())

    def max(self, x: float) -> float:
        return self._reduce(x, None if self.dist is None else self.dist.ReduceOp.MAX)

    def sum(self, x: float) -> float:
        return self._reduce(x, None if self.dist is None else self.dist.ReduceOp.SUM)

    def emit(self, line: dict) -> None:
        """Rank 0 prints the JSON line; the other ranks print nothing."""
        if self.rank == 0:
            print(json.dumps(line), flush=True)

    def close(self) -> None:
        if self.dist is not None:
            self.dist.destroy_process_group()
            self.dist = None


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--instances", type=int, default=4096)
    ap.add_argument("--seed", type=int, default=2024)
    ap.add_argument("--plain-sample", type=int, default=64)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--quick", action="store_true", help="skip the plain/FP64/e2e/CPU side measurements")
    ap.add_argument("--serve-requests", type=int, default=600, help="requests in the serving run (0: skip)")
    ap.add_argument("--serve-rate", type=float, default=30.0, help="Poisson arrival rate (requests/s)")
    ap.add_argument("--serve-budget-gb", type=float, default=150.0)
    ap.add_argument("--serve-lanes", type=int, default=2, help="server lanes (2: grids <= 128 in their own lane)")
    ap.add_argument("--serve-only", action="store_true")
    ap.add_argument("--saturate", type=int, default=1000,
                    help="requests submitted at once for the serving-capacity run (0: skip)")
    ap.add_argument("--plain-serve-sample", type=int, default=24,
                    help="requests of that burst run through the one-at-a-time plain FP64 drop-in")
    ap.add_argument("--launch-shape", default="",
                    help="CHUNK,BLOCKS_PER_SM instead of the autotuner (e.g. 4096,32; for profiling)")
    ap.add_argument("--no-graph", action="store_true",
                    help="host-driven loops instead of the per-step CUDA graph (for ncu, which cannot profile "
                         "kernels inside graphs with conditional nodes)")
    ap.add_argument("--precision", choices=["dw", "fp64res"], default="dw",
                    help="refinement arithmetic of the headline: double-word (FP32 pairs) or IEEE FP64")
    ap.add_argument("--precond", choices=["alpha_line", "jacobi"], default="alpha_line",
                    help="inner-solve preconditioner of the headline (the other one is measured beside it)")
    ap.add_argument("--oracle-sample", type=int, default=16,
                    help="batch instances stepped by the oracle (SuperLU) for rel_err_vs_oracle (0: skip)")
    return ap.parse_args()


def peak_hbm():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ----------------------------------------------------------------------------- clocks
class Clocks:
    """Samples SM clocks and throttle reasons with nvidia-smi while the timed region runs."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, local: int = 0):
        vis = [v for v in os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",") if v.strip()]
        self.gpu = vis[local] if local < len(vis) else str(local)
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", self.gpu,
                                          f"--query-gpu={self.Q}", "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if parts[3 + k].lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "samples": len(sm),
                "reasons": sorted(reasons)}


# ----------------------------------------------------------------------------- CPU baseline
def _cpu_worker(p):
    """One instance-step of the oracle port: assembly (C restatement) + SuperLU (COLAMD)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle  # checker / CPU baseline only

    t0 = time.perf_counter()
    M5, R = oracle.assemble(p, p.f0)
    x = oracle.solve(p.nx, p.ny, M5, R, "splu")
    return time.perf_counter() - t0, float(x.min())


def cpu_baseline_single(seed, n, seconds):
    """Bounded single-core sample: instances 0, 1, 2, ... for about `seconds` of CPU work."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle  # checker / CPU baseline only

    oracle.build()
    sizes = cases.batch_sizes(n, seed)
    spent, done = 0.0, 0
    while spent < seconds and done < n:
        p = cases.batch_instance(done, seed, DT, sizes[done])
        dt, _ = _cpu_worker(p)
        spent += dt
        done += 1
    cells = sum(a * b for a, b in sizes[:done])
    return {"value": done / spent, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"instances 0..{done - 1} of the batch ({cells} cells) x 1 step each, {spent:.1f} s: "
                      "C restatement of Solver.cc assembly + SuperLU/COLAMD direct solve, one thread"}


def _oracle_steps(args):
    """The oracle (C restatement of the reference's assembly + SuperLU/COLAMD) stepping batch
    instance k from f0 for nsteps steps: the checker of the GPU batch's results."""
    k, seed, size, nsteps = args
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle  # checker / CPU baseline only

    p = cases.batch_instance(k, seed, DT, size)
    return k, oracle.step(p, None, nsteps, solver="splu")


def oracle_errors(seed, sizes, f_gpu, stats, n):
    """Relative L2 error against the oracle for n instances spread over the batch's size range
    (quantiles of the cell count), each stepped by the oracle as many steps as the GPU batch took,
    on all host cores (a spawned pool). Returns the summary and the per-instance records."""
    import multiprocessing as mp

    cells = np.array([x * y for x, y in sizes], dtype=np.int64)
    order = np.argsort(cells, kind="stable")
    pick = sorted({int(order[q]) for q in np.linspace(0, len(order) - 1, n).round().astype(int)})
    jobs = [(k, seed, sizes[k], int(stats[k]["steps"])) for k in pick]
    t0 = time.perf_counter()
    with mp.get_context("spawn").Pool(min(len(jobs), os.cpu_count() or 1)) as pool:
        res = dict(pool.map(_oracle_steps, jobs))
    per = []
    for k in pick:
        ref = res[k]
        per.append({"instance": k, "grid": list(sizes[k]), "steps": int(stats[k]["steps"]),
                    "rel_err": float(np.linalg.norm(f_gpu[k] - ref) / np.linalg.norm(ref)),
                    "min_f": float(stats[k]["min_f"]), "mass_drift": float(stats[k]["mass_drift"])})
    errs = [r["rel_err"] for r in per]
    return {"max": max(errs), "median": statistics.median(errs), "instances": len(per),
            "oracle": "C restatement of Solver.cc assembly + SuperLU/COLAMD, every step from f0",
            "seconds": time.perf_counter() - t0}, per


def run_reference(a):
    """--impl reference: the oracle port on every host core, same config/metric."""
    import multiprocessing as mp

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle  # checker / CPU baseline only

    oracle.build()
    cores = os.cpu_count() or 1
    per_step = max(cores, 8)
    sizes = cases.batch_sizes(a.instances, a.seed)
    nsamples = max(a.warmup, 1) + a.steps
    ks = [(s * per_step + i) % a.instances for s in range(nsamples) for i in range(per_step)]
    probs = {k: cases.batch_instance(k, a.seed, DT, sizes[k]) for k in sorted(set(ks))}
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        def sample(s):
            return pool.map(_cpu_worker, [probs[k] for k in ks[s * per_step:(s + 1) * per_step]])

        for s in range(max(a.warmup, 1)):
            sample(s)
        t0 = time.perf_counter()
        mins = []
        for s in range(max(a.warmup, 1), nsamples):
            mins += [m for _, m in sample(s)]
        wall = time.perf_counter() - t0
    v = per_step * a.steps / wall
    line = {"metric": METRIC, "value": v, "unit": UNIT, "impl": "reference", "n_gpus": a.gpus,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1e3 * wall / a.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded)",
            "config": {"workload": f"batched: {a.instances} instances, nalpha,nE~U[64,256], dt={DT} day; "
                                   f"each bench step = {per_step} instance-steps sampled from the batch",
                       "instances": a.instances, "seed": a.seed},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{per_step} instance-steps per bench step on {cores} processes: C "
                                       "restatement of Solver.cc assembly + SuperLU/COLAMD (Eigen SparseLU "
                                       "stand-in; the reference build needs Eigen/xtensor/HDF5)"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "min_f": min(mins) if mins else None}
    print(json.dumps(line))


# ----------------------------------------------------------------------------- our arm
# Algorithmic bytes per real cell per launch (FP32+refine path): reads + writes of the arrays
# each kernel must touch once (neighbour re-reads served by cache are not counted).
BYTES32 = {
    "assemble": 2 * 8 + 8 * 8 + 4 * (4 + 4) + 4 * 8,  # f, start g, 8 factors -> 4 hi+lo coefs, invD/R/colsum/y
    "resid": 8 + 4 + 8 + 4 * (4 + 4) + 8 + 4,     # y, x, R, hi+lo coefs -> y', r
    "bicg1": 4 * 4 + 4 * 4 + 2 * 4,               # r, p, v, r^, 4 coefs -> p', v'
    "bicg2": 2 * 4 + 4 * 4 + 4,                   # r, v, 4 coefs -> t
    "bicg3": 6 * 4 + 2 * 4,                       # r, v, p, t, r^, x -> x, r
    "polish": 8 + 4 * (4 + 4) + 3 * 8 + 8 + 3 * 8 + 8 + 3 * 8,  # y, hi+lo coefs, R, invD, colsum, f, 3 earlier
                                                            # states, loss factor -> f, history slot, start g
}


# The same for the FP64 drop-in (mode 0): FP64 Krylov vectors and coefficients.
BYTES64 = {
    "assemble": BYTES32["assemble"],              # 8-byte coefficients either way (FP64 or hi+lo)
    "resid": 8 + 8 + 8 + 4 * 8 + 8 + 8,           # y, x, R, coefs -> y', r
    "bicg1": 4 * 8 + 4 * 8 + 2 * 8,               # r, p, v, r^, 4 coefs -> p', v'
    "bicg2": 2 * 8 + 4 * 8 + 8,                   # r, v, 4 coefs -> t
    "bicg3": 6 * 8 + 2 * 8,                       # r, v, p, t, r^, x -> x, r
    "polish": BYTES32["polish"],
}


# The algorithmic bytes per cell of the hot-path analysis, for the assembly: read f, Lxx, Lxy,
# Lyy, UKK, s (48 B), write 5 coefficients and R (48 B). The roofline's `achieved` and `frac` use
# it; the design's own model above (what this layout must move) is reported beside it.
ANALYSIS_BYTES = {"assemble": 96}


# DRAM bytes per processed cell measured by ncu (dram__bytes_read.sum + dram__bytes_write.sum) on the
# 256-instance case of the same kernels (one ncu capture per kernel); traffic grows with the
# cells processed, so a launch's traffic is this figure times the cells it processed.
TRAFFIC32 = {"assemble": 142.5, "bicg1": 27.5, "bicg2": 26.5, "bicg3": 23.2, "resid": 58.1, "polish": 131.5}


def kernel_roofline(b, probs, peak, steps=2, model=None):
    """Per-kernel event timing over `steps` steps; bytes from the cells each kernel processed
    (model: bytes per cell per kernel, BYTES32 by default)."""
    model = BYTES32 if model is None else model
    cells = np.array([p.nx * p.ny for p in probs], dtype=np.float64)
    before = [b.stats(k) for k in range(len(probs))]
    b.enable_timing(True)
    b.step(steps, allow_not_converged=True)
    kt = b.kernel_times()
    b.enable_timing(False)
    after = [b.stats(k) for k in range(len(probs))]
    it = np.array([a["total_iterations"] - c["total_iterations"] for a, c in zip(after, before)], dtype=np.float64)
    rf = np.array([a["total_refinements"] - c["total_refinements"] for a, c in zip(after, before)], dtype=np.float64)
    proc = {"assemble": cells.sum() * steps, "polish": cells.sum() * steps, "resid": (cells * rf).sum(),
            "bicg1": (cells * it).sum(), "bicg2": (cells * it).sum(), "bicg3": (cells * it).sum()}
    out = {}
    for name, (ms, n) in kt.items():
        if name == "solve_coop" and n > 0:  # the refinement loop as one cooperative kernel
            byts = sum(model[k] * proc[k] for k in ("resid", "bicg1", "bicg2", "bicg3"))
            out[name] = {"ms": ms, "launches": int(n), "bytes": byts, "GBps": byts / (ms * 1e-3) / 1e9,
                         "share": 0.0}
        elif name in model and n > 0:
            byts = model[name] * proc[name]
            out[name] = {"ms": ms, "launches": int(n), "bytes": byts, "GBps": byts / (ms * 1e-3) / 1e9,
                         "share": 0.0}
        else:
            out[name] = {"ms": ms, "launches": int(n)}
    total = sum(v["ms"] for k, v in out.items() if not k.startswith("krylov_"))
    for v in out.values():
        v["share"] = v["ms"] / total if total else 0.0
    dom = max((k for k in out if k in model), key=lambda k: out[k]["ms"])
    d = out[dom]
    ach = d["GBps"]
    traffic = (TRAFFIC32[dom] * d["bytes"] / BYTES32[dom] / d["launches"]
               if dom in TRAFFIC32 and model is BYTES32 else None)
    design = ach
    if dom in ANALYSIS_BYTES:
        ach = design * ANALYSIS_BYTES[dom] / model[dom]
    roof = {"bound": "hbm", "kernel": dom, "achieved": ach, "peak": peak[0], "unit": "GB/s",
            "frac": ach / peak[0], "peak_source": peak[1], "traffic": traffic,
            "bytes_per_cell_analysis": ANALYSIS_BYTES.get(dom, model[dom]),
            "achieved_design_model": design, "frac_design_model": design / peak[0],
            "bytes_per_cell_design_model": model[dom],
            "traffic_source": "ncu dram bytes per cell on 256 instances, scaled by the cells processed",
            "bytes_per_launch": d["bytes"] / d["launches"] * (ANALYSIS_BYTES.get(dom, model[dom]) / model[dom]),
            "avg_launch_ms": d["ms"] / d["launches"]}
    return roof, out


SERVE_POOL = 1024  # distinct request problems at most; longer streams reuse them in turn


def serving_requests(nreq, rate, seed):
    """Seeded request stream: Poisson arrivals at `rate`, n log-uniform in [32, 512] (n x n grid),
    steps log-uniform in [10, 2000], seeded D fields, rho and tau per request. Streams longer
    than SERVE_POOL requests draw their problems from SERVE_POOL distinct ones in turn (each
    request keeps its own step count and arrival time), which bounds host memory."""
    rng = np.random.default_rng([seed, 4242])
    arrivals = np.cumsum(rng.exponential(1.0 / rate, size=nreq))
    n = np.rint(np.exp(rng.uniform(np.log(32), np.log(512), size=nreq))).astype(int)
    steps = np.rint(np.exp(rng.uniform(np.log(10), np.log(2000), size=nreq))).astype(int)
    pool = []
    for k in range(min(nreq, SERVE_POOL)):
        r = np.random.default_rng([seed, k, 99])
        pool.append(cases.synthetic_problem(int(n[k]), int(n[k]), DT, seed=seed * 104729 + k,
                                            tau=float(10.0 ** r.uniform(-1, 1)), rho=float(r.uniform(-0.9, 0.9))))
    probs = [pool[k % len(pool)] for k in range(nreq)]
    return arrivals, probs, steps


def run_serving(capi, arrivals, probs, steps, precision, budget_gb, lanes=2):
    """Drives a server in real time: submits each request at its arrival time, ticks, polls.
    Latency = result ready - arrival time (both on the monotonic clock). Two lanes by default:
    grids up to 128 x 128 in their own lane with a quarter of the budget."""
    srv = capi.Server(budget_gb * 1e9, max_slots=4096, max_side=512, precision=precision, lanes=lanes,
                      split_side=128, small_fraction=0.25)
    nreq = len(probs)
    t0 = time.monotonic()
    nxt, live, lat, min_f, not_conv = 0, {}, [], float("inf"), 0
    while len(lat) < nreq:
        now = time.monotonic() - t0
        while nxt < nreq and arrivals[nxt] <= now:
            live[srv.submit(probs[nxt], int(steps[nxt]))] = nxt
            nxt += 1
        info = srv.info()
        if info["resident"] == 0 and info["waiting"] == 0:
            if nxt < nreq:
                time.sleep(max(0.0, arrivals[nxt] - (time.monotonic() - t0)))
            continue
        if srv.tick() > 0:
            for rid in srv.completed_ids():
                r = srv.poll(rid, want_f=False)
                k = live.pop(rid)
                _, st, ts, td = r
                lat.append(td - (t0 + arrivals[k]))
                min_f = min(min_f, st["min_f"])
                not_conv += int(st["status"] != 0)
    wall = time.monotonic() - t0
    info = srv.info()
    srv.close()
    lat = np.array(lat) * 1e3
    return {"requests": nreq, "lanes": lanes, "p50_ms": float(np.percentile(lat, 50)),
            "p99_ms": float(np.percentile(lat, 99)),
            "mean_ms": float(lat.mean()), "wall_s": wall,
            "instance_steps_per_s": info["instance_steps"] / wall,
            "cell_steps_per_s": float(sum(p.nx * p.ny * int(s) for p, s in zip(probs, steps))) / wall,
            "requests_per_s": nreq / wall, "ticks": info["ticks"], "busy_s": info["busy_seconds"],
            "tick_split_s": {k: info[k + "_seconds"] for k in ("admit", "lists", "step", "collect")},
            "min_f": min_f, "not_converged": not_conv, "device_gb": info["device_bytes"] / 1e9}


def run_saturation(capi, probs, steps, precision, budget_gb, lanes=2):
    """Serving capacity: every request is submitted at once (arrivals far above what the device
    drains) and the server ticks until all have completed. Reports the drain throughput
    (instance-steps and cell-steps per second over the whole drain) and the same over the time
    in which the first 90 % of the instance-steps were done (the last requests, the longest
    ones, finish with few instances resident), with p50/p99 completion times."""
    srv = capi.Server(budget_gb * 1e9, max_slots=4096, max_side=512, precision=precision, lanes=lanes,
                      split_side=128, small_fraction=0.25)
    total_is = int(sum(int(n) for n in steps))
    total_cs = float(sum(p.nx * p.ny * int(n) for p, n in zip(probs, steps)))
    t0 = time.monotonic()
    live = {srv.submit(p, int(n)): k for k, (p, n) in enumerate(zip(probs, steps))}
    done_t, trace = [], []
    while live:
        if srv.tick() > 0:
            for rid in srv.completed_ids():
                srv.poll(rid, want_f=False)
                live.pop(rid)
                done_t.append(time.monotonic() - t0)
        trace.append((time.monotonic() - t0, srv.info()["instance_steps"]))
    wall = time.monotonic() - t0
    info = srv.info()
    srv.close()
    t90 = next(t for t, n in trace if n >= 0.9 * total_is)
    ct = np.array(done_t) * 1e3
    return {"requests": len(probs), "lanes": lanes, "wall_s": wall,
            "instance_steps_per_s": total_is / wall, "cell_steps_per_s": total_cs / wall,
            "instance_steps_per_s_first90": 0.9 * total_is / t90, "t90_s": t90,
            "completion_p50_ms": float(np.percentile(ct, 50)), "completion_p99_ms": float(np.percentile(ct, 99)),
            "ticks": info["ticks"], "device_gb": info["device_bytes"] / 1e9}


def run_plain_dropin(capi, probs, steps):
    """The one-at-a-time plain FP64 drop-in on the same requests: one sayram_create per request,
    its steps, the result read back, destroyed; instance-steps and cell-steps per second."""
    t0 = time.monotonic()
    for p, n in zip(probs, steps):
        s = capi.Solver(p, precision=capi.FP64)
        s.step(int(n), allow_not_converged=True)
        s.f()
        s.close()
    wall = time.monotonic() - t0
    return {"requests": len(probs), "wall_s": wall,
            "instance_steps_per_s": sum(int(n) for n in steps) / wall,
            "cell_steps_per_s": float(sum(p.nx * p.ny * int(n) for p, n in zip(probs, steps))) / wall}


def run_1024(capi, peak):
    """The single-instance 1024 x 1024 configuration (dt = 1e-2): device-timed steps/s of the
    plain FP64 drop-in and of the double-word path, each with both inner-solve preconditioners
    and the launch shape the autotuner picks for it;
    iterations of the last step; the step's HBM fraction (model bytes of every kernel launch in two
    host-loop steps, per step, over the graph step's time); the agreement of the results."""
    p = cases.synthetic_problem(1024, 1024, DT, seed=11)
    out = {"grid": "1024 x 1024", "dt": DT, "peak_GBps": peak[0]}
    fs = {}
    for name, prec, model in (("fp64", capi.FP64, BYTES64), ("fp32_refine_dw", capi.FP32_REFINE_DW, BYTES32)):
        for pcn, pc in (("alpha_line", capi.PRECOND_ALPHA_LINE), ("jacobi", capi.PRECOND_JACOBI)):
            s = capi.Solver(p, precision=prec, precond=pc)
            shape = s.autotune(2)  # restores the state: the run below starts from f0
            s.step(4)
            s.record_event(0)
            s.step(10)
            s.record_event(1)
            ms = s.elapsed_ms(0, 1) / 10
            st = s.get_stats()
            fs[(name, pcn)] = s.f()
            _, kern = kernel_roofline(s, [p], peak, steps=2, model=model)
            step_bytes = sum(v.get("bytes", 0.0) for v in kern.values()) / 2
            kms = sum(v["ms"] for k, v in kern.items() if not k.startswith("krylov_")) / 2
            out[f"{name}/{pcn}"] = {
                "steps_per_s": 1e3 / ms, "ms_per_step": ms, "iterations_last_step": st["iterations"],
                "launch_shape": {"cells_per_chunk": shape[0], "blocks_per_sm": shape[1]},
                "refinements_last_step": st["refinements"], "rel_residual": st["rel_residual"],
                "model_bytes_per_step": step_bytes, "hbm_frac_step": step_bytes / (ms * 1e-3) / 1e9 / peak[0],
                "kernel_ms_per_step": kms, "hbm_frac_kernels": step_bytes / (kms * 1e-3) / 1e9 / peak[0],
                "kernels": {k: {"ms": v["ms"] / 2, "launches": v["launches"] / 2} for k, v in kern.items()}}
            s.close()
    ref = fs[("fp64", "alpha_line")]
    out["rel_err_vs_fp64_alpha_line"] = {f"{n}/{c}": float(np.linalg.norm(f - ref) / np.linalg.norm(ref))
                                         for (n, c), f in fs.items() if (n, c) != ("fp64", "alpha_line")}
    return out


def run_ours(a, R: Ranks):
    from sayram2d_gb300 import build, capi

    build.build()
    capi.load()
    t0 = time.perf_counter()
    # weak scaling: every rank steps a.instances instances of a batch of world * a.instances
    probs = cases.batch_shard(a.instances, a.seed, DT, R.rank, R.world)
    gen_s = time.perf_counter() - t0
    ncells = int(sum(p.nx * p.ny for p in probs))
    prec = capi.FP32_REFINE_DW if a.precision == "dw" else capi.FP32_REFINE
    other = capi.FP32_REFINE if a.precision == "dw" else capi.FP32_REFINE_DW
    pc = capi.PRECOND_ALPHA_LINE if a.precond == "alpha_line" else capi.PRECOND_JACOBI
    b = capi.Batch(probs, precision=prec, use_graph=0 if a.no_graph else 1, device=R.local, precond=pc)
    t0 = time.perf_counter()
    if a.launch_shape:
        b.set_launch_shape(*[int(v) for v in a.launch_shape.split(",")])
        shape = b.launch_shape()
    else:
        shape = b.autotune(2)
    tune_s = time.perf_counter() - t0
    for _ in range(a.warmup):
        b.step(1, allow_not_converged=True)
    l0 = b.launches()
    clk = Clocks(R.local)
    clk.start()
    R.barrier()  # every rank's warm-up has finished (b.step synchronises its stream)
    b.record_event(0)
    rc = b.step(a.steps, allow_not_converged=True)
    b.record_event(1)
    ms = R.max(b.elapsed_ms(0, 1))  # elapsed_ms synchronises on the end event
    R.barrier()
    clocks = clk.stop()
    launches = int(R.sum(b.launches() - l0))
    value = R.world * a.instances * a.steps / (ms * 1e-3)
    peak = peak_hbm()
    roof, kern = kernel_roofline(b, probs, peak)
    tail = kern.get("krylov_tail10", {"ms": 0.0, "share": 0.0})
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": R.world, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": ms / a.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+dw" if a.precision == "dw" else "f32+f64",
            "data": "synthetic (seeded)",
            "config": {"workload": f"batched FP32 Krylov + refinement: {a.instances} instances, nalpha,nE~U[64,256], "
                                   f"rho~U[-0.9,0.9], tau~logU[0.1,10] d, dt={DT} day, refined to rel residual 1e-11",
                       "instances": R.world * a.instances, "instances_per_gpu": a.instances,
                       "parallelism": (f"{R.world} ranks, one GPU each, instance-sharded (no data-path collective)"
                                       if R.world > 1 else "one GPU"),
                       "cells": int(R.sum(ncells)), "seed": a.seed,
                       "precision": ("fp32_refine_dw: FP32 Krylov, double-word (FP32-pair, ~48-bit) residual/"
                                     "refinement/assembly/checks" if a.precision == "dw" else
                                     "fp32_refine: FP32 Krylov, IEEE FP64 residual/refinement/assembly/checks"),
                       "precond": ("alpha-line 4-cell blocks (left-preconditioned BiCGSTAB)" if a.precond == "alpha_line"
                                   else "Jacobi scaling only"),
                       "l2": f"working set {b.device_bytes() / 1e9:.1f} GB >> 129 MB L2 (no flush needed)",
                       "launch_shape": {"cells_per_chunk": shape[0], "blocks_per_sm": shape[1],
                                        "autotune_s": tune_s, "candidates": b.tuning_log()}},
            "gpu_launches": int(launches), "roofline": roof, "kernels": kern, "clocks": clocks,
            "krylov_tail10": {"share_of_step_kernel_time": tail["share"],
                              "what": "BiCGSTAB iterations in which < 10 % of the instances were still iterating "
                                      "(host-loop timing steps)"},
            "status_last_step": rc, "setup_s": {"generate": gen_s}}
    # accuracy: per-instance stats and rel L2 against the batched FP64 path after the same steps
    st = [b.stats(k) for k in range(len(probs))]
    nsteps_done = st[0]["steps"]
    line["min_f"] = min(s["min_f"] for s in st)
    line["max_mass_drift"] = max(s["mass_drift"] for s in st)
    line["max_rel_residual"] = max(s["rel_residual"] for s in st)
    line["not_converged"] = int(sum(1 for s in st if s["status"] != 0))
    line["mean_inner_iterations"] = sum(s["total_iterations"] for s in st) / max(1, sum(s["steps"] for s in st))
    line["mean_refinements"] = sum(s["total_refinements"] for s in st) / max(1, sum(s["steps"] for s in st))
    for key, red in (("min_f", min), ("max_mass_drift", max), ("max_rel_residual", max)):
        line[key] = -R.max(-line[key]) if red is min else R.max(line[key])
    line["not_converged"] = int(R.sum(line["not_converged"]))
    if not a.quick:
        f32 = [b.f(k) for k in range(len(probs))]
        # e2e through the public C-ABI with pinned host buffers (every rank its own shard)
        L = capi.load()
        nbytes = 8 * ncells
        hin = L.sayram_host_alloc(nbytes)
        hout = L.sayram_host_alloc(nbytes)
        arr_in = np.ctypeslib.as_array((__import__("ctypes").c_double * ncells).from_address(hin))
        arr_in[:] = np.concatenate([f.ravel() for f in f32])
        b.step_host(1, hin, hout, allow_not_converged=True)  # warm
        e2e_steps = max(3, a.steps // 2)
        R.barrier()
        t0 = time.perf_counter()
        for s in range(e2e_steps):
            src, dst = (hout, hin) if s % 2 == 0 else (hin, hout)
            b.step_host(1, src, dst, allow_not_converged=True)
        wall = R.max(time.perf_counter() - t0)
        L.sayram_host_free(hin)
        L.sayram_host_free(hout)
        line["e2e"] = {"value": R.world * a.instances * e2e_steps / wall, "unit": UNIT,
                       "h2d_bytes_per_step": int(R.sum(nbytes)), "d2h_bytes_per_step": int(R.sum(nbytes)),
                       "steps": e2e_steps, "api": "sayram_batch_step_host (pinned host f in/out every step)"}
        b.close()
    if not a.quick and R.world == 1:
        # the other refinement arithmetic on the same batch (device-timed, a few steps)
        bo = capi.Batch(probs, precision=other)
        bo.autotune(2)
        for _ in range(2):
            bo.step(1, allow_not_converged=True)
        bo.record_event(0)
        bo.step(5, allow_not_converged=True)
        bo.record_event(1)
        mso = bo.elapsed_ms(0, 1) / 5
        name_o = "fp32_refine_fp64_residual" if a.precision == "dw" else "fp32_refine_dw"
        line[name_o] = {"value": a.instances / (mso * 1e-3), "unit": UNIT, "ms_per_step": mso}
        bo.close()
        # the headline arithmetic with the other inner-solve preconditioner
        pco = capi.PRECOND_JACOBI if pc == capi.PRECOND_ALPHA_LINE else capi.PRECOND_ALPHA_LINE
        bp = capi.Batch(probs, precision=prec, precond=pco)
        bp.autotune(2)
        for _ in range(2):
            bp.step(1, allow_not_converged=True)
        i0 = sum(bp.stats(k)["total_iterations"] for k in range(len(probs)))
        bp.record_event(0)
        bp.step(5, allow_not_converged=True)
        bp.record_event(1)
        msp = bp.elapsed_ms(0, 1) / 5
        i1 = sum(bp.stats(k)["total_iterations"] for k in range(len(probs)))
        line["other_precond"] = {"precond": "jacobi" if pco == capi.PRECOND_JACOBI else "alpha_line",
                                 "value": a.instances / (msp * 1e-3), "unit": UNIT, "ms_per_step": msp,
                                 "mean_inner_iterations": (i1 - i0) / (5 * len(probs))}
        bp.close()
        # batched FP64 on the same batch, same number of steps -> accuracy + precision gain
        b64 = capi.Batch(probs, precision=capi.FP64)
        b64.autotune(1)
        b64.step(nsteps_done - 1, allow_not_converged=True)
        b64.record_event(0)
        b64.step(1, allow_not_converged=True)
        b64.record_event(1)
        ms64 = b64.elapsed_ms(0, 1)
        errs = []
        for k in range(len(probs)):
            g = b64.f(k)
            errs.append(float(np.linalg.norm(f32[k] - g) / np.linalg.norm(g)))
        b64.close()
        line["rel_err_vs_fp64"] = {"max": max(errs), "median": statistics.median(errs),
                                   "reference": "batched FP64 GPU path (matches the oracle to <=1e-10)"}
        line["batched_fp64"] = {"value": a.instances / (ms64 * 1e-3), "unit": UNIT, "ms_per_step": ms64}
        # plain FP64 drop-in, one instance after another
        ns = min(a.plain_sample, len(probs))
        tot = 0.0
        for k in range(ns):
            s = capi.Solver(probs[k], precision=capi.FP64)
            s.update()
            s.record_event(0)
            s.step(2)
            s.record_event(1)
            tot += s.elapsed_ms(0, 1) * 1e-3
            s.close()
        plain = 2 * ns / tot
        line["plain_fp64"] = {"value": plain, "unit": UNIT,
                              "sample": f"first {ns} instances, 2 steps each, one sayram_create per instance"}
        line["speedup_vs_plain_fp64"] = value / plain
        line["cpu_baseline"] = cpu_baseline_single(a.seed, a.instances, a.cpu_seconds)
        if a.oracle_sample > 0:
            # the same leg checks the timed batch's results against the oracle (not timed)
            line["rel_err_vs_oracle"], line["oracle_sample"] = oracle_errors(
                a.seed, cases.batch_sizes(a.instances, a.seed), f32, st, a.oracle_sample)
        line["config_1024"] = run_1024(capi, peak)
    b.close()
    if a.serve_requests > 0 and R.world == 1:
        arr, sprobs, ssteps = serving_requests(a.serve_requests, a.serve_rate, a.seed)
        cfg = (f"{a.serve_requests} Poisson requests at {a.serve_rate}/s, n~logU[32,512] (n x n), "
               f"steps~logU[10,2000], dt={DT} day, HBM budget {a.serve_budget_gb} GB")
        line["serving"] = {"config": cfg, "precision": "fp32_refine_dw",
                           **run_serving(capi, arr, sprobs, ssteps, capi.FP32_REFINE_DW, a.serve_budget_gb, a.serve_lanes)}
        if not a.quick:
            line["serving_plain_fp64"] = {"config": cfg, "precision": "fp64",
                                          **run_serving(capi, arr, sprobs, ssteps, capi.FP64, a.serve_budget_gb, a.serve_lanes)}
    if a.saturate > 0 and R.world == 1 and not a.quick:
        line["serving_capacity"] = saturation(capi, a)
    R.emit(line)


def saturation(capi, a):
    """Serving capacity on a burst of --saturate requests of the serving distribution (seeded):
    dw serving, plain FP64 serving and the one-at-a-time plain FP64 drop-in (on the burst's first
    --plain-serve-sample requests); the ratios use cell-steps/s, which does not depend on which
    requests a sample holds."""
    _, bprobs, bsteps = serving_requests(a.saturate, 1.0, a.seed + 1)
    out = {"config": f"{a.saturate} requests submitted at once, n~logU[32,512] (n x n), steps~logU[10,2000], "
                     f"dt={DT} day, HBM budget {a.serve_budget_gb} GB, {a.serve_lanes} lanes"}
    out["fp32_refine_dw"] = run_saturation(capi, bprobs, bsteps, capi.FP32_REFINE_DW, a.serve_budget_gb, a.serve_lanes)
    out["fp64"] = run_saturation(capi, bprobs, bsteps, capi.FP64, a.serve_budget_gb, a.serve_lanes)
    m = min(a.plain_serve_sample, a.saturate)
    out["plain_fp64_dropin"] = {"sample": f"first {m} requests of the burst", **run_plain_dropin(capi, bprobs[:m], bsteps[:m])}
    cs = lambda k: out[k]["cell_steps_per_s"]
    out["speedup_cell_steps"] = {"dw_serving_vs_plain_dropin": cs("fp32_refine_dw") / cs("plain_fp64_dropin"),
                                 "dw_serving_vs_fp64_serving": cs("fp32_refine_dw") / cs("fp64"),
                                 "fp64_serving_vs_plain_dropin": cs("fp64") / cs("plain_fp64_dropin")}
    return out


def run_serve_only(a):
    """Only the serving measurement (one JSON line): both precisions, the request stream of
    --serve-requests / --serve-rate / --serve-budget-gb."""
    from sayram2d_gb300 import build, capi

    build.build()
    capi.load()
    arr, sprobs, ssteps = serving_requests(a.serve_requests, a.serve_rate, a.seed)
    cfg = (f"{a.serve_requests} Poisson requests at {a.serve_rate}/s, n~logU[32,512] (n x n), "
           f"steps~logU[10,2000], dt={DT} day, HBM budget {a.serve_budget_gb} GB, "
           f"{min(a.serve_requests, SERVE_POOL)} distinct problems")
    line = {"metric": "serving latency p50/p99 (ms) and throughput", "unit": "ms", "n_gpus": 1,
            "data": "synthetic (seeded)", "config": {"workload": cfg}}
    line["serving"] = {"precision": "fp32_refine_dw",
                       **run_serving(capi, arr, sprobs, ssteps, capi.FP32_REFINE_DW, a.serve_budget_gb, a.serve_lanes)}
    if not a.quick:
        line["serving_plain_fp64"] = {"precision": "fp64",
                                      **run_serving(capi, arr, sprobs, ssteps, capi.FP64, a.serve_budget_gb, a.serve_lanes)}
    print(json.dumps(line))


def main():
    a = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if a.gpus != world:
        raise SystemExit(f"--gpus {a.gpus} with WORLD_SIZE={world}: launch N > 1 GPUs with torchrun "
                         "(one process per GPU)")
    if a.warmup < 3 and a.impl == "ours":
        a.warmup = 3
    if a.impl == "reference":
        # the reference's CPU path runs once, on rank 0's host cores; other ranks do no work
        if int(os.environ.get("RANK", "0")) == 0:
            run_reference(a)
        return
    if a.serve_only:
        if int(os.environ.get("RANK", "0")) == 0:
            run_serve_only(a)
        return
    R = Ranks()
    try:
        run_ours(a, R)
    finally:
        R.close()


if __name__ == "__main__":
    main()
