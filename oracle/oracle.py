"""TEST INFRASTRUCTURE: Python front end of the CPU oracle (the checker, never the product).

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may import this
module.  It wraps

  * ``_build/libppfv_oracle.so`` -- ppfv_oracle.c, the C restatement of Sayram-2D's
    ``Solver::update()`` (source/Solver.cc:270-290) with a banded direct LU;
  * scipy's SuperLU (``splu``, COLAMD column ordering) -- the same supernodal-LU/COLAMD family
    as the reference's ``Eigen::SparseLU<SpMat, COLAMDOrdering<int>>`` (Solver.h:35), used as a
    second direct solver and for grids where banded LU is too slow;
  * ``_ref/libsayram_ref.so`` when it exists -- the reference's own Solver.cc/Mesh.cc built
    against the shim headers (Makefile target ``ref``), used to pin the restatement.

Problems are any object with the attributes of ``cases.Problem``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libppfv_oracle.so")
REF_PATH = os.path.join(HERE, "_ref", "libsayram_ref.so")
REF_CASE_PATH = os.path.join(HERE, "_ref", "libsayram_case_ref.so")

_dp = ctypes.POINTER(ctypes.c_double)
_lock = threading.Lock()
_lib = None
_ref = None
_ref_case = None


class _OrcProblem(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int), ("ny", ctypes.c_int),
        ("x_edges", _dp), ("y_edges", _dp),
        ("dt", ctypes.c_double),
        ("bc", ctypes.c_int * 4),
        ("G", _dp), ("Dxx", _dp), ("Dxy", _dp), ("Dyy", _dp), ("inv_tau", _dp),
        ("dir", _dp * 4),
    ]


class _OrcDTable(ctypes.Structure):
    _fields_ = [("na", ctypes.c_int), ("ne", ctypes.c_int), ("alpha0_deg", _dp), ("E", _dp),
                ("Daa", _dp), ("Dap", _dp), ("Dpp", _dp)]


def build(force: bool = False) -> str:
    """Compiles the C restatement (make in this directory)."""
    if force or not os.path.exists(LIB_PATH):
        subprocess.run(["make", "-C", HERE, "-s", "all"], check=True)
    return LIB_PATH


ROOT_NOTE = os.path.join(HERE, "_ref", "REFERENCE_ROOT")


def reference_root() -> str | None:
    """The reference's source tree (the directory holding ``source/`` and ``D/``): the
    ``SAYRAM_REFERENCE`` environment variable, else the tree the last :func:`build_ref` compiled;
    None when neither names an existing tree (callers skip what needs the reference)."""
    cands = [os.environ.get("SAYRAM_REFERENCE", "")]
    if os.path.exists(ROOT_NOTE):
        with open(ROOT_NOTE) as fh:
            cands.append(fh.read().strip())
    for c in cands:
        if c and os.path.isdir(os.path.join(c, "source")):
            return c
    return None


def build_ref(reference_root_dir: str | None = None) -> str | None:
    """Compiles the reference's own solver sources when they are present (the given tree, else
    :func:`reference_root`) and records the tree in ``_ref/REFERENCE_ROOT``; returns the path."""
    root = reference_root_dir or reference_root()
    if not root or not os.path.isdir(os.path.join(root, "source")):
        return REF_PATH if os.path.exists(REF_PATH) else None
    subprocess.run(["make", "-C", HERE, "-s", "ref", f"REF={root}"], check=True)
    with open(ROOT_NOTE, "w") as fh:
        fh.write(os.path.abspath(root) + "\n")
    return REF_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(LIB_PATH)
            P = ctypes.POINTER(_OrcProblem)
            L.orc_vertex_f.argtypes = [P, _dp, _dp]
            L.orc_face_coeffs.argtypes = [P, _dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp]
            L.orc_assemble.argtypes = [P, _dp, _dp, _dp]
            L.orc_assemble_bound.argtypes = [P, _dp, _dp, _dp, _dp]
            L.orc_assemble_bound.restype = ctypes.c_int
            L.orc_solve.argtypes = [ctypes.c_int, ctypes.c_int, _dp, _dp, _dp]
            L.orc_step.argtypes = [P, _dp, ctypes.c_int]
            L.orc_dtable_fields.argtypes = [ctypes.c_int, ctypes.c_int, _dp, _dp, ctypes.POINTER(_OrcDTable),
                                            _dp, _dp, _dp]
            L.orc_dtable_fields.restype = ctypes.c_int
            for fn in (L.orc_vertex_f, L.orc_face_coeffs, L.orc_assemble, L.orc_solve, L.orc_step):
                fn.restype = ctypes.c_int
            _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_dp)


class _Packed:
    """Keeps contiguous float64 copies alive while the C struct points at them."""

    def __init__(self, prob):
        c = lambda a: np.ascontiguousarray(a, dtype=np.float64)
        self.keep = [c(prob.x_edges), c(prob.y_edges), c(prob.G), c(prob.Dxx), c(prob.Dxy),
                     c(prob.Dyy), c(prob.inv_tau)]
        self.dirs = [None if d is None else c(d) for d in prob.dirichlet]
        s = _OrcProblem()
        s.nx, s.ny, s.dt = int(prob.nx), int(prob.ny), float(prob.dt)
        xe, ye, G, Dxx, Dxy, Dyy, it = self.keep
        s.x_edges, s.y_edges = _ptr(xe), _ptr(ye)
        s.G, s.Dxx, s.Dxy, s.Dyy, s.inv_tau = _ptr(G), _ptr(Dxx), _ptr(Dxy), _ptr(Dyy), _ptr(it)
        for k in range(4):
            s.bc[k] = int(prob.bc[k])
            s.dir[k] = _dp() if self.dirs[k] is None else _ptr(self.dirs[k])
        self.s = s


def _check(rc, what):
    if rc != 0:
        raise RuntimeError(f"oracle {what} failed with code {rc}")


def vertex_f(prob, f):
    P = _Packed(prob)
    f = np.ascontiguousarray(f, dtype=np.float64)
    vf = np.empty((prob.nx + 1, prob.ny + 1))
    _check(lib().orc_vertex_f(ctypes.byref(P.s), _ptr(f), _ptr(vf)), "vertex_f")
    return vf


def face_coeffs(prob, f, i, j, inbr):
    """(a_sigma_A, a_sigma_B, a_sigma) of cell (i, j) toward neighbour direction inbr."""
    P = _Packed(prob)
    f = np.ascontiguousarray(f, dtype=np.float64)
    out = np.empty(3)
    _check(lib().orc_face_coeffs(ctypes.byref(P.s), _ptr(f), i, j, inbr, _ptr(out)), "face_coeffs")
    return out


def assemble(prob, f):
    """M as five diagonals (5, N) [diag, W, E, S, N] and R (N,), system order K = j*nx + i."""
    P = _Packed(prob)
    f = np.ascontiguousarray(f, dtype=np.float64)
    N = prob.nx * prob.ny
    M5 = np.empty((5, N))
    R = np.empty(N)
    _check(lib().orc_assemble(ctypes.byref(P.s), _ptr(f), _ptr(M5), _ptr(R)), "assemble")
    return M5, R


def assemble_bound(prob, f):
    """(M5, R, B5): B5 is each entry's forward-error scale (its formula on term magnitudes)."""
    P = _Packed(prob)
    f = np.ascontiguousarray(f, dtype=np.float64)
    N = prob.nx * prob.ny
    M5, B5 = np.empty((5, N)), np.empty((5, N))
    R = np.empty(N)
    _check(lib().orc_assemble_bound(ctypes.byref(P.s), _ptr(f), _ptr(M5), _ptr(R), _ptr(B5)), "assemble_bound")
    return M5, R, B5


def to_csc(nx, ny, M5):
    """scipy CSC matrix of the five diagonals (the reference's SpMat is column-major)."""
    import scipy.sparse as sp

    N = nx * ny
    K = np.arange(N)
    i = K % nx
    rows, cols, vals = [K], [K], [M5[0]]
    for d, off, ok in ((1, -1, i > 0), (2, 1, i < nx - 1), (3, -nx, K - nx >= 0), (4, nx, K + nx < N)):
        rows.append(K[ok]); cols.append(K[ok] + off); vals.append(M5[d][ok])
    return sp.csc_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(N, N))


def solve(nx, ny, M5, R, solver="banded"):
    """Direct solve of M x = R: banded LU without pivoting, or SuperLU with COLAMD."""
    if solver == "splu":
        import scipy.sparse.linalg as spla

        return spla.splu(to_csc(nx, ny, M5), permc_spec="COLAMD").solve(np.asarray(R, dtype=np.float64))
    M5 = np.ascontiguousarray(M5, dtype=np.float64)
    R = np.ascontiguousarray(R, dtype=np.float64)
    x = np.empty(nx * ny)
    _check(lib().orc_solve(nx, ny, _ptr(M5), _ptr(R), _ptr(x)), "solve")
    return x


def residual_ext(nx, ny, M5, R, x):
    """R - M x in extended precision (numpy longdouble: 64-bit significand on x86-64 and 113-bit
    on aarch64), from the five diagonals; returned as float64 with its norm ratio ||r|| / ||R||."""
    ld = np.longdouble
    d = np.asarray(M5, dtype=ld)
    xv = np.asarray(x, dtype=ld)
    N = nx * ny
    K = np.arange(N)
    i = K % nx
    y = d[0] * xv
    for row, off, ok in ((1, -1, i > 0), (2, 1, i < nx - 1), (3, -nx, K - nx >= 0), (4, nx, K + nx < N)):
        idx = K[ok]
        y[idx] += d[row][idx] * xv[idx + off]
    r = np.asarray(R, dtype=ld) - y
    nr = float(np.sqrt(np.sum(r * r)) / np.sqrt(np.sum(np.asarray(R, dtype=ld) ** 2)))
    return r.astype(np.float64), nr


def alpha_line_solver(nx, ny, M5):
    """Solves the alpha-line (i-direction) tridiagonal part of M: diagonal plus the W/E couplings
    of each E row (Thomas elimination of every row at once, scipy.linalg.solve_banded)."""
    import scipy.linalg as sla

    N = nx * ny
    ab = np.zeros((3, N))
    ab[1] = M5[0]
    K = np.arange(N)
    i = K % nx
    ab[0, 1:] = np.where(i[:-1] < nx - 1, M5[2][:-1], 0.0)  # row K, column K+1 (east)
    ab[2, :-1] = np.where(i[1:] > 0, M5[1][1:], 0.0)       # row K+1, column K (west)
    return lambda b: sla.solve_banded((1, 1), ab, b, check_finite=False)


def solve_tight(nx, ny, M5, R, x0=None, rtol=1e-15, max_refine=12):
    """M x = R to a relative residual of ``rtol`` measured in extended precision, or to the
    rounding floor of a float64 x when that is higher (refinement stops once a pass gains less
    than 4x): iterative refinement whose correction equations are solved by BiCGSTAB with the
    alpha-line preconditioner (scipy), each to 1e-9. Returns (x, relative residual, inner
    iterations). The
    direct solvers above give the same x to the conditioning of M; this one reaches grids where
    they are too slow (1024 x 1024 in a few seconds per step)."""
    import scipy.sparse.linalg as spla

    N = nx * ny
    A = to_csc(nx, ny, M5).tocsr()
    P = spla.LinearOperator((N, N), matvec=alpha_line_solver(nx, ny, M5))
    x = np.zeros(N) if x0 is None else np.array(x0, dtype=np.float64, copy=True)
    its = [0]

    def count(_):
        its[0] += 1

    r, rel = residual_ext(nx, ny, M5, R, x)
    for _ in range(max_refine):
        if rel <= rtol:
            break
        d, _info = spla.bicgstab(A, r, rtol=1e-9, atol=0.0, maxiter=5000, M=P, callback=count)
        xn = x + d
        rn, reln = residual_ext(nx, ny, M5, R, xn)
        if not reln < rel:
            break  # at the rounding floor of a float64 x (about u * ||M|| ||x|| / ||R||)
        stalled = reln > 0.25 * rel
        x, r, rel = xn, rn, reln
        if stalled:
            break
    return x, rel, its[0]


def sys_to_field(nx, ny, x):
    """System order K = j*nx + i -> alpha-major (nx, ny) (the copy back of Solver.cc:280-284)."""
    return np.ascontiguousarray(np.asarray(x).reshape(ny, nx).T)


def field_to_sys(f):
    return np.ascontiguousarray(np.asarray(f).T).reshape(-1)


def step(prob, f=None, nsteps=1, solver="banded"):
    """nsteps of Solver::update from f (default prob.f0); returns the new alpha-major f. solver:
    "banded" (C banded LU), "splu" (SuperLU/COLAMD) or "tight" (solve_tight, started from f)."""
    f = np.array(prob.f0 if f is None else f, dtype=np.float64, copy=True)
    if solver == "tight":
        for _ in range(nsteps):
            M5, R = assemble(prob, f)
            x, _, _ = solve_tight(prob.nx, prob.ny, M5, R, field_to_sys(f))
            f = sys_to_field(prob.nx, prob.ny, x)
        return f
    if solver == "banded":
        P = _Packed(prob)
        _check(lib().orc_step(ctypes.byref(P.s), _ptr(f), int(nsteps)), "step")
        return f
    for _ in range(nsteps):
        M5, R = assemble(prob, f)
        f = sys_to_field(prob.nx, prob.ny, solve(prob.nx, prob.ny, M5, R, solver))
    return f


def column_sums(nx, ny, M5):
    """1^T M per column (the discrete conservation law 1^T M f = 1^T R)."""
    return np.asarray(to_csc(nx, ny, M5).sum(axis=0)).ravel()


# ----------------------------------------------------------------------------- reference build
def ref_lib():
    global _ref
    with _lock:
        if _ref is None:
            if not os.path.exists(REF_PATH):
                return None
            L = ctypes.CDLL(REF_PATH)
            L.ref_run.argtypes = [ctypes.c_int, ctypes.c_int, _dp, _dp, ctypes.c_double,
                                  ctypes.POINTER(ctypes.c_int), _dp, _dp, _dp, _dp, _dp, _dp,
                                  ctypes.POINTER(_dp), ctypes.c_int, _dp, _dp, _dp]
            L.ref_run.restype = ctypes.c_int
            L.ref_last_error.restype = ctypes.c_char_p
            _ref = L
    return _ref


def ref_run(prob, nsteps):
    """Runs the reference's own Solver (oracle/_ref). Returns (M5, R, f): the matrix and RHS that
    its constructor assembles from f0, and f after nsteps updates."""
    L = ref_lib()
    if L is None:
        raise RuntimeError("reference build not available (make -C oracle ref)")
    P = _Packed(prob)
    f0 = np.ascontiguousarray(prob.f0, dtype=np.float64)
    N = prob.nx * prob.ny
    M5 = np.empty((5, N))
    R = np.empty(N)
    f = np.empty((prob.nx, prob.ny))
    bc = (ctypes.c_int * 4)(*[int(b) for b in prob.bc])
    dirs = (_dp * 4)(*[P.s.dir[k] for k in range(4)])
    rc = L.ref_run(prob.nx, prob.ny, P.s.x_edges, P.s.y_edges, prob.dt, bc, P.s.G, P.s.Dxx,
                   P.s.Dxy, P.s.Dyy, P.s.inv_tau, _ptr(f0), dirs, int(nsteps), _ptr(M5), _ptr(R), _ptr(f))
    if rc != 0:
        raise RuntimeError("reference run failed: " + L.ref_last_error().decode())
    return M5, R, f


# ----------------------------------------------------------------------------- D table
def _pack_table(t):
    c = lambda a: np.ascontiguousarray(a, dtype=np.float64)
    keep = [c(t.alpha0_deg), c(t.E), c(t.Daa), c(t.Dap), c(t.Dpp)]
    s = _OrcDTable(len(keep[0]), len(keep[1]), *[_ptr(a) for a in keep])
    return s, keep


def dtable_fields(x_edges, y_edges, table):
    """Dxx, Dxy, Dyy (alpha-major) interpolated from a D table at the cell centres, as the
    Albert_Young cases' constructD does (orc_dtable_fields)."""
    xe = np.ascontiguousarray(x_edges, dtype=np.float64)
    ye = np.ascontiguousarray(y_edges, dtype=np.float64)
    nx, ny = len(xe) - 1, len(ye) - 1
    s, keep = _pack_table(table)
    out = [np.empty((nx, ny)) for _ in range(3)]
    _check(lib().orc_dtable_fields(nx, ny, _ptr(xe), _ptr(ye), ctypes.byref(s), *[_ptr(o) for o in out]),
           "dtable_fields")
    return tuple(out)


def ref_case_lib():
    global _ref_case
    with _lock:
        if _ref_case is None:
            if not os.path.exists(REF_CASE_PATH):
                return None
            L = ctypes.CDLL(REF_CASE_PATH)
            L.ref_case.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp, _dp, ctypes.c_double,
                                   ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int, _dp, _dp,
                                   _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp,
                                   ctypes.POINTER(ctypes.c_int), _dp]
            L.ref_case.restype = ctypes.c_int
            L.ref_case_last_error.restype = ctypes.c_char_p
            _ref_case = L
    return _ref_case


def ref_case(which, x_edges, y_edges, dt, Emin, Emax, table):
    """Runs the reference's own Albert_Young (which=0) or Albert_Young_LC (1) case on the grid and
    D table (oracle/_ref). Returns G, Dxx, Dxy, Dyy, inv_tau, f0 (alpha-major), bc[4] and the
    Dirichlet vertex values per side (None for zero-flux sides)."""
    L = ref_case_lib()
    if L is None:
        raise RuntimeError("reference case build not available (make -C oracle ref)")
    xe = np.ascontiguousarray(x_edges, dtype=np.float64)
    ye = np.ascontiguousarray(y_edges, dtype=np.float64)
    nx, ny = len(xe) - 1, len(ye) - 1
    s, keep = _pack_table(table)
    out = {k: np.empty((nx, ny)) for k in ("G", "Dxx", "Dxy", "Dyy", "inv_tau", "f0")}
    bc = (ctypes.c_int * 4)()
    dirv = np.zeros(2 * (ny + 1) + 2 * (nx + 1))
    rc = L.ref_case(int(which), nx, ny, _ptr(xe), _ptr(ye), float(dt), float(Emin), float(Emax), s.na, s.ne,
                    s.alpha0_deg, s.E, s.Daa, s.Dap, s.Dpp, *[_ptr(out[k]) for k in out], bc, _ptr(dirv))
    if rc != 0:
        raise RuntimeError("reference case failed: " + L.ref_case_last_error().decode())
    out["bc"] = [int(b) for b in bc]
    offs = np.cumsum([0, ny + 1, ny + 1, nx + 1, nx + 1])
    out["dirichlet"] = [dirv[offs[k]:offs[k + 1]].copy() if out["bc"][k] == 0 else None for k in range(4)]
    return out
