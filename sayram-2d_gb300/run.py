"""The reference's main program (Sayram-2D ``source/main.cc:39-95``) on the GPU path: an ini file in,
the HDF5 output file out.

``run(ini)`` does what ``main`` does with a parameter file:

* ``Parameters`` (``Parameters.cc:3-17``): reads the ini (:func:`cases.read_ini`, with the
  reference's ``nsteps`` rounding and ``dt = T / nsteps``), creates ``./output/<run_id>/`` and
  copies the ini file there as ``<run_id>.ini``;
* ``Albert_Young eq(paras, m)`` (``main.cc:49``): :func:`case_of` -- G, f0, the BCs and the loss
  term on the host, the D table from ``D/<dID>.h5`` (``Albert_Young_IO.cc:17-36``, read by the
  library's HDF5 reader) interpolated on the device (``Albert_Young.cc:94-134``); the loss-cone
  variant ``Albert_Young_LC`` and the seeded ``[synthetic]`` case are chosen by the ini;
* ``Solver solver(m, &eq)`` (``main.cc:51``): the drop-in :class:`capi.Solver`;
* ``HighFive::File(..._data.h5, Overwrite)`` (``main.cc:56-57``): :class:`capi.H5File`;
* ``/alpha0 = x / pi * 180`` and ``/logEN = y - ln E0`` (``main.cc:59-66``), ``/f/0`` (``:74``);
* the time loop (``main.cc:77-84``): ``save_every_step`` steps, then ``/f/<k>``; the steps between
  two saves run as one device call, since both reference cases have time-independent
  coefficients (``Albert_Young.cc:62``, ``Albert_Young_LC.cc:76``: ``update`` does nothing);
* ``/t = linspace(0, T, nplots + 1)`` (``main.cc:86-89``).

As in the reference, a step that ends above its residual target is not an error (the reference
never checks ``SparseLU::info()``, ``Solver.cc:277``); the solver's statistics report it.
"""
from __future__ import annotations

import math
import os
import shutil
import sys
from typing import Optional

import numpy as np

from . import capi, cases

PRECISIONS = {
    "fp64": capi.FP64,
    "fp32_refine": capi.FP32_REFINE,
    "fp32_refine_dw": capi.FP32_REFINE_DW,
}


def output_dir(rp: cases.RunParams, root: str = ".") -> str:
    return os.path.join(root, "output", rp.run_id)  # Parameters.cc:7


def output_file(rp: cases.RunParams, root: str = ".") -> str:
    return os.path.join(output_dir(rp, root), rp.run_id + "_data.h5")  # main.cc:56


def write_axes(h5: "capi.H5File", problem: cases.Problem) -> None:
    """/alpha0 and /logEN from the cell centres (main.cc:59-66; Mesh.cc:50, 62)."""
    x = 0.5 * (problem.x_edges[:-1] + problem.x_edges[1:])
    y = 0.5 * (problem.y_edges[:-1] + problem.y_edges[1:])
    h5.write("/alpha0", x / cases.PI * 180.0)
    h5.write("/logEN", y - math.log(cases.E0))


def case_of(rp: cases.RunParams, root: str = "."):
    """The Equation an ini describes (``Albert_Young eq(paras, m)``, main.cc:49): its Problem and,
    for the Albert_Young cases, the D table read from ``D/<dID>.h5`` under ``root``
    (Albert_Young_IO::read_D, Albert_Young_IO.cc:17-36), else None. A missing or unreadable table
    is an error, as in the reference (its HDF5 read throws)."""
    prob = cases.problem_from_params(rp)
    if rp.equation == cases.SYNTHETIC:
        return prob, None
    path = cases.dtable_path(rp, root)
    if not os.path.isfile(path):
        raise FileNotFoundError(f"{rp.equation} run {rp.run_id!r}: D table {path} not found")
    return prob, capi.load_dtable(path)


def run(ini_path: str, root: str = ".", problem: Optional[cases.Problem] = None,
        precision: Optional[str] = None) -> str:
    """Runs the case an ini file describes and returns the path of its HDF5 output.

    The case is the ini's (:func:`cases.read_ini`): an Albert_Young case takes its D table from
    ``<root>/D/<dID>.h5`` and interpolates it on the device (``constructD``,
    Albert_Young.cc:112-134); a ``[synthetic]`` ini generates its seeded fields. ``problem``
    replaces the case entirely (same grid expected; no D table is read then); ``precision``
    replaces the ini's ``[solver] precision``."""
    rp = cases.read_ini(ini_path)
    if problem is not None:
        prob, table = problem, None
    else:
        prob, table = case_of(rp, root)
    if (prob.nx, prob.ny) != (rp.nalpha0, rp.nE):
        raise ValueError(f"problem grid {prob.nx}x{prob.ny} differs from the ini's {rp.nalpha0}x{rp.nE}")
    name = precision or rp.precision
    if name not in PRECISIONS:
        raise ValueError(f"precision {name!r}: expected one of {sorted(PRECISIONS)}")
    out = output_dir(rp, root)
    os.makedirs(out, exist_ok=True)
    shutil.copyfile(ini_path, os.path.join(out, rp.run_id + ".ini"))  # Parameters.cc:10-16
    solver = capi.Solver(prob, precision=PRECISIONS[name], tol=rp.tol)
    if table is not None:
        try:
            solver.set_dtable(table)
        except Exception:
            solver.close()
            raise
    path = output_file(rp, root)
    try:
        with capi.H5File(path) as h5:
            write_axes(h5, prob)
            h5.write("/f/0", solver.f())
            for k in range(1, rp.nplots + 1):
                solver.step(rp.save_every_step, allow_not_converged=True)
                h5.write(f"/f/{k}", solver.f())
            h5.write("/t", np.linspace(0.0, rp.T, rp.nplots + 1))
    finally:
        solver.close()
    return path


def main(argv=None) -> int:
    """Command-line entry with main.cc's argument handling (Parameters.cc:19-33): at most one
    argument, the parameter file, ``p.ini`` by default. Prints the output file's path."""
    argv = sys.argv[1:] if argv is None else argv
    if len(argv) > 1:
        print("This program takes at most one argument: the parameter file name.", file=sys.stderr)
        return 1
    print(run(argv[0] if argv else "p.ini"))
    return 0
