"""Generates the golden fixtures in this directory from the reference's OWN solver sources.

Sayram-2D's source/Solver.cc and source/Mesh.cc are compiled unmodified against the project's
Eigen/xtensor shim headers (``make -C oracle ref`` -> oracle/_ref/libsayram_ref.so) and driven by
oracle/ref_harness.cc. For every case this script stores the inputs, the matrix M (five
diagonals, system order) and right-hand side R that the reference assembles from f0, and f after
1 and ``nsteps`` updates. The config-0 case (90 x 90, 1000 steps) stores only outputs; its inputs
are regenerated from the seeded generator (an input checksum guards against drift).

Run here (where the reference sources exist):  python tests/golden/make_golden.py
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


def main():
    oracle.build()
    if oracle.build_ref() is None:
        raise SystemExit("the reference sources are needed to generate fixtures")
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
