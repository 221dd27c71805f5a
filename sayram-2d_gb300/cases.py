"""Cases: the data a Sayram-2D ``Equation`` supplies to the solver, as plain arrays.

The reference's solver reads, per cell, ``G, Dxx, Dxy, Dyy, inv_tau`` (``source/Equation.h:44-50``),
the initial state ``init_f`` (``Equation.h:55``), the boundary types ``bc_type(side)``
(``Equation.h:52``) and Dirichlet vertex values ``dirichlet_vertex_value(side, i, j, t)``
(``Equation.h:60-65``).  A :class:`Problem` carries exactly those, evaluated on a grid, so that the
GPU library, the oracle and the tests all see the same inputs.

Layouts follow the reference: per-cell fields are ``(nx, ny)`` alpha-major (``i*ny + j``, the
xtensor row-major order of ``Equation::G_`` etc.); Dirichlet vertex values are indexed by ``j`` in
``[0, ny]`` for XMIN/XMAX and by ``i`` in ``[0, nx]`` for YMIN/YMAX (``Solver.cc:398-419``).

Generators:
  * :func:`synthetic_problem` -- the seeded synthetic physics used for every benchmark workload
    (Albert & Young 2005 geometry and G, smooth seeded D fields, loss term, f0 and BCs).
  * :func:`albert_young_problem` -- the ``Albert_Young`` case's G, f0 and BCs
    (``source/Cases/Albert_Young.{h,cc}``) with seeded D fields standing in for the HDF5 table.
  * :func:`albert_young_lc_problem` -- the loss-cone variant (``source/Cases/Albert_Young_LC.cc``).
"""
from __future__ import annotations

import configparser
import dataclasses
import math
import os
from typing import List, Optional, Sequence

import numpy as np

EPS = float(np.finfo(np.float64).eps)  # gEPS, source/common.h:38
PI = 3.141592653589793238462  # gPI, common.h:39
E0 = 0.511875  # gE0 [MeV], common.h:41 (gC = 1)
RE = 6371000.0  # gRE, common.h:43

XMIN, XMAX, YMIN, YMAX = 0, 1, 2, 3  # BoundaryID, source/BCTypes.h:13
DIRICHLET, ZEROFLUX = 0, 1  # BCType, source/BCTypes.h:16


@dataclasses.dataclass
class Problem:
    """One solver instance: grid, time step, coefficients, initial state and BCs."""

    nx: int
    ny: int
    x_edges: np.ndarray  # (nx+1,)
    y_edges: np.ndarray  # (ny+1,)
    dt: float
    bc: List[int]  # [XMIN, XMAX, YMIN, YMAX]
    G: np.ndarray  # (nx, ny) alpha-major, float64
    Dxx: np.ndarray
    Dxy: np.ndarray
    Dyy: np.ndarray
    inv_tau: np.ndarray
    f0: np.ndarray
    dirichlet: List[Optional[np.ndarray]]  # per side; None for zero-flux sides
    name: str = ""

    @property
    def ncells(self) -> int:
        return self.nx * self.ny

    def validate(self) -> None:
        """The checks of Grid2D::validate (Grid2D.h:44-67) and Mesh (Mesh.cc:37-63), plus shapes."""
        if self.nx < 1 or self.ny < 1:
            raise ValueError("Grid2D: x_edges/y_edges must have size >= 2.")
        if self.x_edges.shape != (self.nx + 1,) or self.y_edges.shape != (self.ny + 1,):
            raise ValueError("Mesh: edges size mismatch.")
        if not np.all(np.diff(self.x_edges) > 0):
            raise ValueError("Grid2D: x_edges must be strictly increasing.")
        if not np.all(np.diff(self.y_edges) > 0):
            raise ValueError("Grid2D: y_edges must be strictly increasing.")
        if not (self.dt > 0):
            raise ValueError("dt must be positive")
        for name in ("G", "Dxx", "Dxy", "Dyy", "inv_tau", "f0"):
            a = getattr(self, name)
            if a.shape != (self.nx, self.ny) or a.dtype != np.float64:
                raise ValueError(f"{name} must be float64 of shape (nx, ny)")
        for s in range(4):
            if self.bc[s] not in (DIRICHLET, ZEROFLUX):
                raise ValueError("unknown BC type")
            if self.bc[s] == DIRICHLET:
                v = self.dirichlet[s]
                n = self.ny + 1 if s in (XMIN, XMAX) else self.nx + 1
                if v is None or np.asarray(v).shape != (n,):
                    raise ValueError("Dirichlet BC: missing value.")  # Solver.cc:393


# ----------------------------------------------------------------------------- physics helpers
def e2p(E):
    """Momentum from kinetic energy (utils.h:12-14), in units with gC = 1."""
    return np.sqrt(E * (E + 2 * E0))


def p2e(p):
    """Kinetic energy from momentum (utils.h:7-9)."""
    return np.sqrt(p * p + E0 * E0) - E0


def dlogE_dp(logE):
    """d(log E)/dp (utils.h:17-20)."""
    E = np.exp(logE)
    return e2p(E) / (E * (E + E0))


def uniform_edges(n: int, lo: float, hi: float) -> np.ndarray:
    """Uniform edges as main.cc:20-37 builds them: lo + d*i with d = (hi-lo)/n."""
    d = (hi - lo) / float(n)
    return lo + d * np.arange(n + 1, dtype=np.float64)


def _centres(edges: np.ndarray) -> np.ndarray:
    return 0.5 * (edges[:-1] + edges[1:])  # Mesh.cc:50, 62


def _ay_G(A, Y):
    """G of Albert_Young::calculate_G (Albert_Young.h:42-45)."""
    t = 1.30 - 0.56 * np.sin(A)
    return e2p(np.exp(Y)) ** 2 * t * np.sin(A) * np.cos(A) / dlogE_dp(Y)


def _smooth_field(rng, xi, eta):
    """A smooth seeded field in [0, 1] over normalised coordinates xi, eta in [0, 1]."""
    ka, ke = rng.uniform(0.5, 2.0, size=2)
    pa, pe = rng.uniform(0.0, 2 * np.pi, size=2)
    return 0.5 + 0.25 * np.sin(2 * np.pi * ka * xi + pa) + 0.25 * np.sin(2 * np.pi * ke * eta + pe)


def synthetic_D(rng, A, Y, rho: float, lo: float = -6.0, hi: float = -2.0):
    """Seeded D fields: log-uniform magnitudes 10^lo..10^hi per day shaped by smooth fields and a
    sin(alpha0) pitch-angle profile; Dxy = rho*sqrt(Dxx*Dyy) with |rho| < 1 keeps D positive
    definite."""
    xi = (A - A.min()) / max(A.max() - A.min(), 1e-300)
    eta = (Y - Y.min()) / max(Y.max() - Y.min(), 1e-300)
    Dxx = 10.0 ** (lo + (hi - lo) * _smooth_field(rng, xi, eta)) * np.sin(A)
    Dyy = 10.0 ** (lo + (hi - lo) * _smooth_field(rng, xi, eta)) * np.sin(A)
    Dxy = rho * np.sqrt(Dxx * Dyy)
    return Dxx, Dxy, Dyy


def synthetic_problem(
    nalpha: int,
    nE: int,
    dt: float,
    seed: int,
    tau: Optional[float] = 1.0,
    rho: Optional[float] = None,
    alpha0_min_deg: float = 5.0,
    alpha0_max_deg: float = 90.0,
    Emin: float = 0.2,
    Emax: float = 5.0,
    D_range=(-6.0, -2.0),
    x_edges: Optional[np.ndarray] = None,
    y_edges: Optional[np.ndarray] = None,
    bc: Optional[Sequence[int]] = None,
) -> Problem:
    """The seeded synthetic case of the benchmark workloads.

    Grid: alpha0 uniform in [alpha0_min, alpha0_max] (radians), log E uniform in
    [log Emin, log Emax] (main.cc:20-37). G from Albert_Young (Albert_Young.h:42-45).
    D: :func:`synthetic_D` with rho drawn uniform in [-0.9, 0.9] unless given. Loss term
    inv_tau = 1/tau everywhere (0 if tau is None). f0 = exp(-(E-0.2)/0.1)*sin(alpha0) + eps.
    BCs: XMIN (loss cone) Dirichlet 0; XMAX (90 deg) zero flux; YMIN Dirichlet f0(alpha0, Emin) at
    the vertices; YMAX Dirichlet 0 (as Albert_Young.h:52-62). ``x_edges``/``y_edges`` replace the
    uniform grids (any strictly increasing edges, as Grid2D accepts); ``bc`` replaces the BC types
    (Dirichlet sides keep the values above; an XMAX Dirichlet side is held at f0(alpha0_max, E) at
    its vertices).
    """
    rng = np.random.default_rng(seed)
    if rho is None:
        rho = float(rng.uniform(-0.9, 0.9))
    xe = uniform_edges(nalpha, alpha0_min_deg * PI / 180, alpha0_max_deg * PI / 180) if x_edges is None \
        else np.asarray(x_edges, dtype=np.float64)
    ye = uniform_edges(nE, math.log(Emin), math.log(Emax)) if y_edges is None \
        else np.asarray(y_edges, dtype=np.float64)
    x, y = _centres(xe), _centres(ye)
    A, Y = np.meshgrid(x, y, indexing="ij")
    G = _ay_G(A, Y)
    Dxx, Dxy, Dyy = synthetic_D(rng, A, Y, rho, *D_range)
    inv_tau = np.full((nalpha, nE), 0.0 if tau is None else 1.0 / tau)
    E = np.exp(Y)
    f0 = np.exp(-(E - 0.2) / 0.1) * np.sin(A) + EPS
    bc = list(bc) if bc is not None else [DIRICHLET, ZEROFLUX, DIRICHLET, DIRICHLET]
    Ev = np.exp(ye)
    side_vals = [
        np.zeros(nE + 1),
        np.exp(-(Ev - 0.2) / 0.1) * np.sin(xe[-1]) + EPS,
        np.exp(-(Emin - 0.2) / 0.1) * np.sin(xe) + EPS,
        np.zeros(nalpha + 1),
    ]
    dirichlet = [side_vals[s] if bc[s] == DIRICHLET else None for s in range(4)]
    prob = Problem(
        nalpha, nE, xe, ye, float(dt), bc,
        G, Dxx, Dxy, Dyy, inv_tau, f0, dirichlet, name=f"synthetic-{nalpha}x{nE}-s{seed}",
    )
    prob.validate()
    return prob


def albert_young_problem(nalpha: int, nE: int, dt: float, seed: int = 0, rho: float = 0.5,
                         alpha0_min_deg: float = 5.0, Emin: float = 0.2, Emax: float = 5.0,
                         D=None, alpha0_max_deg: float = 90.0) -> Problem:
    """Albert_Young's G, f0 and BCs (Albert_Young.h:37-62, Albert_Young.cc:42-92) on main.cc's
    uniform grid (main.cc:20-37). D is (Dxx, Dxy, Dyy) at the cell centres if given (for example
    interpolated from a :class:`DTable`; zeros when the device interpolates the table afterwards,
    ``sayram_set_dtable``); otherwise seeded synthetic fields stand in for the HDF5 table."""
    rng = np.random.default_rng(seed)
    xe = uniform_edges(nalpha, alpha0_min_deg * PI / 180, alpha0_max_deg * PI / 180)
    ye = uniform_edges(nE, math.log(Emin), math.log(Emax))
    A, Y = np.meshgrid(_centres(xe), _centres(ye), indexing="ij")

    def init_f(a, logE):  # Albert_Young::calculate_init_f
        p = e2p(np.exp(logE))
        return np.exp(-(np.exp(logE) - 0.2) / 0.1) * (np.sin(a) - np.sin(5 * PI / 180)) / (p * p) + EPS

    Dxx, Dxy, Dyy = synthetic_D(rng, A, Y, rho) if D is None else (np.asarray(d, dtype=np.float64) for d in D)
    dirichlet = [np.zeros(nE + 1), None, init_f(xe, math.log(Emin)), np.zeros(nalpha + 1)]
    prob = Problem(nalpha, nE, xe, ye, float(dt), [DIRICHLET, ZEROFLUX, DIRICHLET, DIRICHLET],
                   _ay_G(A, Y), Dxx, Dxy, Dyy, np.zeros((nalpha, nE)), init_f(A, Y), dirichlet,
                   name=f"albert-young-{nalpha}x{nE}")
    prob.validate()
    return prob


def bounce_period(a0, p, L):
    """Albert_Young_LC::bounce_period (Albert_Young_LC.cc:150-160), in days."""
    T0, T1 = 1.3802, 0.7405
    yv = np.sin(a0)
    Ty = T0 - 0.5 * (T0 - T1) * (yv + np.sqrt(yv))
    return 4 * L * RE * ((E0 + p2e(p))) / p * Ty / (3e8 * 3600 * 24)


def albert_young_lc_problem(nalpha: int, nE: int, dt: float, seed: int = 0, rho: float = 0.5,
                            Emin: float = 0.2, Emax: float = 5.0, D=None, alpha0_min_deg: float = 0.0,
                            alpha0_max_deg: float = 90.0) -> Problem:
    """The loss-cone case (Albert_Young_LC.{h,cc}): alpha0 from 0 deg (the ini's alpha0min), zero
    flux at both alpha0 sides, inv_tau = 4/bounce period inside the loss cone (L = 4.5), Dirichlet
    in E; D as in :func:`albert_young_problem`."""
    rng = np.random.default_rng(seed)
    xe = uniform_edges(nalpha, alpha0_min_deg * PI / 180, alpha0_max_deg * PI / 180)
    ye = uniform_edges(nE, math.log(Emin), math.log(Emax))
    A, Y = np.meshgrid(_centres(xe), _centres(ye), indexing="ij")

    def init_f(a, logE):  # Albert_Young_LC::calculate_init_f
        p = e2p(np.exp(logE))
        return np.exp(-(np.exp(logE) - 0.2) / 0.1) * np.sin(a) / (p * p) + EPS

    L = 4.5
    alpha0lc = math.asin((L ** 5 * (4 * L - 3)) ** -0.25)
    p = e2p(np.exp(Y))
    inv_tau = np.where(A < alpha0lc, 4.0 / bounce_period(A, p, L), 0.0)
    Dxx, Dxy, Dyy = synthetic_D(rng, A, Y, rho) if D is None else (np.asarray(d, dtype=np.float64) for d in D)
    dirichlet = [None, None, init_f(xe, math.log(Emin)), np.zeros(nalpha + 1)]
    prob = Problem(nalpha, nE, xe, ye, float(dt), [ZEROFLUX, ZEROFLUX, DIRICHLET, DIRICHLET],
                   _ay_G(A, Y), Dxx, Dxy, Dyy, inv_tau, init_f(A, Y), dirichlet,
                   name=f"albert-young-lc-{nalpha}x{nE}")
    prob.validate()
    return prob


@dataclasses.dataclass
class DTable:
    """A diffusion-coefficient table as the Albert_Young cases read it from D/<dID>.h5
    (Albert_Young_IO.cc:17-36): /alpha0 in degrees, /E, and /Daa, /Dap, /Dpp of shape
    (len(alpha0), len(E)). The cases interpolate it bilinearly in alpha0 and log E, assuming both
    axes uniform (only the end points are used, Albert_Young.cc:94-110)."""

    alpha0_deg: np.ndarray
    E: np.ndarray
    Daa: np.ndarray
    Dap: np.ndarray
    Dpp: np.ndarray


def synthetic_dtable(seed: int, n_alpha: int = 46, n_E: int = 31, alpha0_max_deg: float = 90.0,
                     Emin: float = 0.1, Emax: float = 10.0, rho: float = 0.6) -> DTable:
    """Seeded stand-in for an Albert-Young D file: smooth positive Daa, Dpp whose converted
    values (x 22643/p^2 etc.) land near 1e-6..1e-2 per day, and Dap = rho' sqrt(Daa Dpp) with a
    smooth |rho'| <= |rho| < 1, so every interpolated D stays positive definite."""
    rng = np.random.default_rng([seed, 91])
    a = np.linspace(0.0, alpha0_max_deg, n_alpha)
    E = np.exp(np.linspace(math.log(Emin), math.log(Emax), n_E))
    A, LE = np.meshgrid(a * PI / 180, np.log(E), indexing="ij")
    xi = A / max(A.max(), 1e-300)
    eta = (LE - LE.min()) / max(LE.max() - LE.min(), 1e-300)
    Daa = 10.0 ** (-9.0 + 3.0 * _smooth_field(rng, xi, eta)) * (0.05 + np.sin(A))
    Dpp = 10.0 ** (-9.5 + 3.0 * _smooth_field(rng, xi, eta)) * (0.05 + np.sin(A))
    Dap = rho * (0.5 + 0.5 * _smooth_field(rng, xi, eta)) * np.sqrt(Daa * Dpp)
    return DTable(a, E, Daa, Dap, Dpp)


def stretched_edges(n: int, lo: float, hi: float, a: float) -> np.ndarray:
    """Non-uniform, strictly increasing edges: lo + (hi-lo)*(u + a*sin(2 pi u)/(2 pi)), |a| < 1."""
    u = np.arange(n + 1, dtype=np.float64) / n
    e = lo + (hi - lo) * (u + a * np.sin(2 * np.pi * u) / (2 * np.pi))
    e[0], e[-1] = lo, hi
    return e


# ----------------------------------------------------------------------------- ini front end
SYNTHETIC, ALBERT_YOUNG, ALBERT_YOUNG_LC = "synthetic", "Albert_Young", "Albert_Young_LC"
EQUATIONS = (SYNTHETIC, ALBERT_YOUNG, ALBERT_YOUNG_LC)


@dataclasses.dataclass
class RunParams:
    """The [basic]/[diagnostics]/[diffusion_coefficients] keys of Parameters::read_inp_file
    (Parameters.cc:35-65) plus the [case], [synthetic] and [solver] sections this project adds.

    ``equation`` is the Equation the run builds: ``Albert_Young`` (what main.cc:49 builds, with D
    interpolated from ``D/<dID>.h5``), ``Albert_Young_LC`` (its loss-cone variant) or
    ``synthetic`` (the seeded benchmark case)."""

    run_id: str
    nalpha0: int
    nE: int
    alpha0_min_deg: float
    alpha0_max_deg: float
    Emin: float
    Emax: float
    T: float
    nsteps: int
    nplots: int
    save_every_step: int
    seed: int = 0
    tau: Optional[float] = 1.0
    rho: Optional[float] = None
    precision: str = "fp64"
    tol: float = 1e-12
    equation: str = SYNTHETIC
    dID: Optional[str] = None

    @property
    def dt(self) -> float:
        return self.T / self.nsteps  # Parameters.h:44, after the rounding below


def read_ini(path: str) -> RunParams:
    """Reads an ini file with the reference's semantics: nsteps is rounded down to a multiple of
    nplots (Parameters.cc:58-60) and dt = T / nsteps.

    Which Equation it describes: ``[case] equation`` when given; otherwise ``synthetic`` when the
    file has a ``[synthetic]`` section, and an Albert_Young case when it names a D table
    (``[diffusion_coefficients] dID``, Parameters.cc:63): ``Albert_Young_LC`` when alpha0 starts
    at 0 (the loss-cone grid of the reference's ``p_AlbertYoungLC.ini``), ``Albert_Young``
    otherwise (the reference's ``p.ini``). A file with neither is refused: it never silently
    becomes a synthetic case."""
    cp = configparser.ConfigParser(inline_comment_prefixes=("#", ";"))
    with open(path) as fh:
        cp.read_file(fh)
    b = cp["basic"]
    nsteps = int(float(b["nsteps"]))
    nplots = int(cp["diagnostics"]["nplots"])
    save_every = nsteps // nplots
    syn = cp["synthetic"] if cp.has_section("synthetic") else {}
    sol = cp["solver"] if cp.has_section("solver") else {}
    dc = cp["diffusion_coefficients"] if cp.has_section("diffusion_coefficients") else {}
    tau = syn.get("tau", "1.0")
    rho = syn.get("rho", None)
    dID = dc.get("dID", None)
    dID = dID.strip() if dID is not None and dID.strip() else None
    alpha0_min = float(b["alpha0min"])
    if cp.has_section("case") and cp["case"].get("equation", "").strip():
        equation = cp["case"]["equation"].strip()
        if equation not in EQUATIONS:
            raise ValueError(f"{path}: [case] equation = {equation!r}: expected one of {list(EQUATIONS)}")
    elif cp.has_section("synthetic"):
        equation = SYNTHETIC
    elif dID is not None:
        equation = ALBERT_YOUNG_LC if alpha0_min == 0.0 else ALBERT_YOUNG
    else:
        raise ValueError(f"{path}: no case to run: the file has neither a [synthetic] section nor "
                         "[diffusion_coefficients] dID (the D table of the Albert_Young cases)")
    if equation != SYNTHETIC and dID is None:
        raise ValueError(f"{path}: {equation} needs [diffusion_coefficients] dID (its D table)")
    return RunParams(
        run_id=b["run_id"], nalpha0=int(b["nalpha0"]), nE=int(b["nE"]),
        alpha0_min_deg=alpha0_min, alpha0_max_deg=float(b["alpha0max"]),
        Emin=float(b["Emin"]), Emax=float(b["Emax"]), T=float(b["T"]),
        nsteps=save_every * nplots, nplots=nplots, save_every_step=save_every,
        seed=int(syn.get("seed", 0)), tau=None if str(tau).lower() == "none" else float(tau),
        rho=None if rho is None else float(rho), precision=str(sol.get("precision", "fp64")),
        tol=float(sol.get("tol", 1e-12)), equation=equation, dID=dID,
    )


def dtable_path(rp: RunParams, root: str = ".") -> str:
    """Where the Albert_Young cases read their D table: ``D/<dID>.h5`` relative to the working
    directory (Albert_Young_IO.cc:19); ``root`` stands for that directory."""
    if rp.dID is None:
        raise ValueError(f"run {rp.run_id!r} names no D table")
    return os.path.join(root, "D", rp.dID + ".h5")


def problem_from_params(rp: RunParams) -> Problem:
    """The Problem an ini file describes. For the Albert_Young cases the D fields are left zero:
    they come from the D table, interpolated on the device after the solver is created
    (``Solver.set_dtable``, as ``run.run`` does)."""
    if rp.equation == SYNTHETIC:
        return synthetic_problem(rp.nalpha0, rp.nE, rp.dt, rp.seed, tau=rp.tau, rho=rp.rho,
                                 alpha0_min_deg=rp.alpha0_min_deg, alpha0_max_deg=rp.alpha0_max_deg,
                                 Emin=rp.Emin, Emax=rp.Emax)
    zero = np.zeros((rp.nalpha0, rp.nE))
    mk = albert_young_problem if rp.equation == ALBERT_YOUNG else albert_young_lc_problem
    return mk(rp.nalpha0, rp.nE, rp.dt, Emin=rp.Emin, Emax=rp.Emax, D=(zero, zero, zero),
              alpha0_min_deg=rp.alpha0_min_deg, alpha0_max_deg=rp.alpha0_max_deg)


# ----------------------------------------------------------------------------- batch workloads
def batch_sizes(n_instances: int, seed: int, lo: int = 64, hi: int = 256):
    """(nalpha, nE) per instance, each uniform in [lo, hi] (the batched workload)."""
    rng = np.random.default_rng(seed)
    return [(int(a), int(e)) for a, e in rng.integers(lo, hi + 1, size=(n_instances, 2))]


def batch_instance(k: int, seed: int, dt: float, size) -> Problem:
    """Instance k of a batch: its own seeded D fields, rho ~ U[-0.9, 0.9], tau log-uniform in
    [0.1, 10] days (independent of the other instances, so any one can be generated alone)."""
    rng = np.random.default_rng([seed, k, 17])
    tau = float(10.0 ** rng.uniform(-1.0, 1.0))
    rho = float(rng.uniform(-0.9, 0.9))
    a, e = size
    return synthetic_problem(int(a), int(e), dt, seed=seed * 7919 + k, tau=tau, rho=rho)


def batch_shard(n_per_rank: int, seed: int, dt: float, rank: int, world: int) -> List[Problem]:
    """Rank `rank`'s share of a batch of world * n_per_rank instances (weak scaling over GPUs):
    global instances [rank * n_per_rank, (rank + 1) * n_per_rank), each generated exactly as
    batch_problems would generate it in the whole batch. Instances are independent, so the
    shards need no exchange."""
    if not (0 <= rank < world):
        raise ValueError(f"rank {rank} outside [0, {world})")
    sizes = batch_sizes(world * n_per_rank, seed)
    return [batch_instance(k, seed, dt, sizes[k]) for k in range(rank * n_per_rank, (rank + 1) * n_per_rank)]


def batch_problems(n_instances: int, seed: int, dt: float, lo: int = 64, hi: int = 256,
                   sizes: Optional[Sequence] = None) -> List[Problem]:
    """Independent seeded instances: sizes uniform in [lo, hi]^2 (see batch_instance)."""
    sizes = sizes if sizes is not None else batch_sizes(n_instances, seed, lo, hi)
    return [batch_instance(k, seed, dt, sizes[k]) for k in range(n_instances)]
