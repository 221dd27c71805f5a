"""ctypes binding of the C-ABI in ``include/sayram_gpu.h`` -- the binding a Python caller of the
reference's ``Solver`` would add -- plus thin classes with the reference's names.

``Solver`` mirrors ``class Solver`` (Sayram-2D ``source/Solver.h:18-26``): construct from a
problem (the Mesh + Equation data), ``update()`` advances one backward-Euler step, ``f()`` returns
the (nx, ny) alpha-major state, ``t()`` the simulated time.  Failures raise ``RuntimeError`` as the
reference throws ``std::runtime_error`` (``Grid2D.h:46-66``, ``Solver.cc:393``).

The compute path is the CUDA library only: if ``_build/libsayram_gpu.so`` is missing or no GPU is
present, construction fails loudly; nothing here falls back to a CPU implementation.
"""
from __future__ import annotations

import ctypes
import os
from typing import List, Optional, Sequence

import numpy as np

from . import build as _build

_dp = ctypes.POINTER(ctypes.c_double)

OK, ERR_ARG, ERR_OOM, ERR_NOT_CONVERGED, ERR_NEGATIVE, ERR_TIMEOUT, ERR_CUDA, ERR_BUDGET, ERR_STATE, ERR_IO = range(10)
FP64, FP32_REFINE, FP32_REFINE_DW = 0, 1, 2
PRECOND_JACOBI, PRECOND_ALPHA_LINE = 0, 1


class sayram_problem(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int), ("ny", ctypes.c_int),
        ("x_edges", _dp), ("y_edges", _dp),
        ("dt", ctypes.c_double),
        ("bc", ctypes.c_int * 4),
        ("G", _dp), ("Dxx", _dp), ("Dxy", _dp), ("Dyy", _dp), ("inv_tau", _dp), ("f0", _dp),
        ("dirichlet", _dp * 4),
    ]


class sayram_options(ctypes.Structure):
    _fields_ = [
        ("precision", ctypes.c_int), ("tol", ctypes.c_double), ("inner_tol", ctypes.c_double),
        ("max_iters", ctypes.c_int), ("max_refine", ctypes.c_int), ("device", ctypes.c_int),
        ("use_graph", ctypes.c_int), ("precond", ctypes.c_int),
    ]


class sayram_stats(ctypes.Structure):
    _fields_ = [
        ("steps", ctypes.c_longlong), ("t", ctypes.c_double), ("status", ctypes.c_int),
        ("refinements", ctypes.c_int), ("iterations", ctypes.c_int),
        ("rel_residual", ctypes.c_double), ("min_f", ctypes.c_double),
        ("clamped", ctypes.c_longlong), ("mass_drift", ctypes.c_double),
        ("total_iterations", ctypes.c_longlong), ("total_refinements", ctypes.c_longlong),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class sayram_dtable(ctypes.Structure):
    _fields_ = [("n_alpha", ctypes.c_int), ("n_energy", ctypes.c_int), ("alpha0_deg", _dp), ("energy", _dp),
                ("Daa", _dp), ("Dap", _dp), ("Dpp", _dp)]


class sayram_server_config(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_double), ("max_slots", ctypes.c_int), ("max_side", ctypes.c_int),
                ("lanes", ctypes.c_int), ("lane_split_side", ctypes.c_int), ("lane_small_fraction", ctypes.c_double),
                ("wait_seconds", ctypes.c_double)]


class sayram_server_info(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_longlong), ("admitted", ctypes.c_longlong), ("completed", ctypes.c_longlong),
                ("waiting", ctypes.c_longlong), ("resident", ctypes.c_longlong), ("ticks", ctypes.c_longlong),
                ("instance_steps", ctypes.c_longlong), ("device_bytes", ctypes.c_double),
                ("arena_cells", ctypes.c_double), ("arena_cells_used", ctypes.c_double),
                ("busy_seconds", ctypes.c_double), ("admit_seconds", ctypes.c_double),
                ("lists_seconds", ctypes.c_double), ("step_seconds", ctypes.c_double),
                ("collect_seconds", ctypes.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


# name -> (restype, argtypes); every symbol the header declares
_P = ctypes.c_void_p
SIGNATURES = {
    "sayram_last_error": (ctypes.c_char_p, []),
    "sayram_version": (ctypes.c_char_p, []),
    "sayram_default_options": (None, [ctypes.POINTER(sayram_options)]),
    "sayram_host_alloc": (ctypes.c_void_p, [ctypes.c_size_t]),
    "sayram_host_free": (None, [ctypes.c_void_p]),
    "sayram_create": (ctypes.c_int, [ctypes.POINTER(sayram_problem), ctypes.POINTER(sayram_options), ctypes.POINTER(_P)]),
    "sayram_update": (ctypes.c_int, [_P]),
    "sayram_step": (ctypes.c_int, [_P, ctypes.c_int]),
    "sayram_t": (ctypes.c_double, [_P]),
    "sayram_get_f": (ctypes.c_int, [_P, _dp]),
    "sayram_set_f": (ctypes.c_int, [_P, _dp]),
    "sayram_set_dirichlet": (ctypes.c_int, [_P, ctypes.c_int, _dp, ctypes.c_int]),
    "sayram_set_coeffs": (ctypes.c_int, [_P, _dp, _dp, _dp, _dp, _dp]),
    "sayram_get_stats": (ctypes.c_int, [_P, ctypes.POINTER(sayram_stats)]),
    "sayram_destroy": (None, [_P]),
    "sayram_batch_create": (ctypes.c_int, [ctypes.POINTER(sayram_problem), ctypes.c_int, ctypes.POINTER(sayram_options), ctypes.POINTER(_P)]),
    "sayram_batch_size": (ctypes.c_int, [_P]),
    "sayram_batch_step": (ctypes.c_int, [_P, ctypes.c_int]),
    "sayram_batch_step_host": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]),
    "sayram_batch_get_f": (ctypes.c_int, [_P, ctypes.c_int, _dp]),
    "sayram_batch_set_f": (ctypes.c_int, [_P, ctypes.c_int, _dp]),
    "sayram_batch_set_dirichlet": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int, _dp, ctypes.c_int]),
    "sayram_batch_set_coeffs": (ctypes.c_int, [_P, ctypes.c_int, _dp, _dp, _dp, _dp, _dp]),
    "sayram_batch_stats": (ctypes.c_int, [_P, ctypes.c_int, ctypes.POINTER(sayram_stats)]),
    "sayram_batch_export_system": (ctypes.c_int, [_P, ctypes.c_int, _dp, _dp]),
    "sayram_batch_device_bytes": (ctypes.c_size_t, [_P]),
    "sayram_batch_stream": (ctypes.c_void_p, [_P]),
    "sayram_batch_record_event": (ctypes.c_int, [_P, ctypes.c_int]),
    "sayram_batch_elapsed_ms": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int, _dp]),
    "sayram_batch_enable_timing": (ctypes.c_int, [_P, ctypes.c_int]),
    "sayram_batch_kernel_times": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_char_p), _dp, ctypes.POINTER(ctypes.c_longlong), ctypes.c_int]),
    "sayram_batch_autotune": (ctypes.c_int, [_P, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]),
    "sayram_batch_set_dtable": (ctypes.c_int, [_P, ctypes.c_int, ctypes.POINTER(sayram_dtable)]),
    "sayram_set_dtable": (ctypes.c_int, [_P, ctypes.POINTER(sayram_dtable)]),
    "sayram_batch_set_launch_shape": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int]),
    "sayram_batch_set_coop": (ctypes.c_int, [_P, ctypes.c_int]),
    "sayram_batch_get_launch_shape": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]),
    "sayram_batch_tuning_log": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int), _dp, ctypes.c_int]),
    "sayram_batch_launches": (ctypes.c_longlong, [_P]),
    "sayram_batch_destroy": (None, [_P]),
    "sayram_instance_bytes": (ctypes.c_size_t, [ctypes.c_int, ctypes.c_int, ctypes.c_int]),
    "sayram_server_create": (ctypes.c_int, [ctypes.POINTER(sayram_server_config), ctypes.POINTER(sayram_options),
                                            ctypes.POINTER(_P)]),
    "sayram_server_submit": (ctypes.c_int, [_P, ctypes.POINTER(sayram_problem), ctypes.c_int,
                                            ctypes.POINTER(ctypes.c_longlong)]),
    "sayram_server_tick": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int)]),
    "sayram_server_poll": (ctypes.c_int, [_P, ctypes.c_longlong, _dp, ctypes.POINTER(sayram_stats), _dp, _dp]),
    "sayram_server_info_get": (ctypes.c_int, [_P, ctypes.POINTER(sayram_server_info)]),
    "sayram_server_completed_ids": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_longlong), ctypes.c_int]),
    "sayram_server_destroy": (None, [_P]),
    "sayram_h5_create": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(_P)]),
    "sayram_h5_write": (ctypes.c_int, [_P, ctypes.c_char_p, _dp, ctypes.c_int, ctypes.POINTER(ctypes.c_longlong)]),
    "sayram_h5_close": (ctypes.c_int, [_P]),
    "sayram_h5_read": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                      ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(_dp)]),
    "sayram_h5_free": (None, [ctypes.c_void_p]),
    "sayram_dtable_load_h5": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(sayram_dtable)]),
    "sayram_dtable_free": (None, [ctypes.POINTER(sayram_dtable)]),
    "sayram_step_noalloc": (ctypes.c_int, [ctypes.POINTER(sayram_problem), ctypes.POINTER(sayram_options),
                                           ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.POINTER(sayram_stats)]),
}

_lib = None


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = False):
    """Loads libsayram_gpu.so (raises if it is missing, unless build_if_missing)."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"{path} is missing: build it first (build.build() / __graft_entry__.build())")
        _build.build()
    L = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def last_error() -> str:
    return (load().sayram_last_error() or b"").decode()


def check(rc: int, what: str, allow=(OK,)) -> int:
    if rc not in allow:
        raise RuntimeError(f"{what} failed (status {rc}): {last_error()}")
    return rc


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def _ptr(a: Optional[np.ndarray]):
    return a.ctypes.data_as(_dp) if a is not None else _dp()


class _Pack:
    """A sayram_problem array and the numpy buffers it points into (kept alive)."""

    def __init__(self, problems: Sequence):
        self.keep: List[np.ndarray] = []
        self.arr = (sayram_problem * len(problems))()
        for k, p in enumerate(problems):
            s = self.arr[k]
            s.nx, s.ny, s.dt = int(p.nx), int(p.ny), float(p.dt)
            for name in ("x_edges", "y_edges", "G", "Dxx", "Dxy", "Dyy", "inv_tau", "f0"):
                a = _f64(getattr(p, name))
                self.keep.append(a)
                setattr(s, name, _ptr(a))
            for side in range(4):
                s.bc[side] = int(p.bc[side])
                d = p.dirichlet[side]
                if d is None:
                    s.dirichlet[side] = _dp()
                else:
                    a = _f64(d)
                    self.keep.append(a)
                    s.dirichlet[side] = _ptr(a)


def options(precision: int = FP64, tol: float = 0.0, inner_tol: float = -1.0, max_iters: int = 500,
            max_refine: int = 6, device: int = 0, use_graph: int = 1,
            precond: Optional[int] = None) -> sayram_options:
    """sayram_default_options with the given fields replaced (precond None: the library's
    default)."""
    o = sayram_options()
    load().sayram_default_options(ctypes.byref(o))
    o.precision, o.tol, o.inner_tol = precision, tol, inner_tol
    o.max_iters, o.max_refine, o.device, o.use_graph = max_iters, max_refine, device, use_graph
    if precond is not None:
        o.precond = precond
    return o


class Batch:
    """Many independent instances advanced by the same device launches (sayram_batch_*)."""

    def __init__(self, problems: Sequence, opts: Optional[sayram_options] = None, **kw):
        L = load()
        self._L = L
        self.problems = list(problems)
        self.shapes = [(int(p.nx), int(p.ny)) for p in self.problems]
        self.offsets = np.cumsum([0] + [a * b for a, b in self.shapes])
        pack = _Pack(self.problems)
        opts = opts if opts is not None else options(**kw)
        h = ctypes.c_void_p()
        check(L.sayram_batch_create(pack.arr, len(self.problems), ctypes.byref(opts), ctypes.byref(h)), "sayram_batch_create")
        self.h = h
        self.opts = opts

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            self._L.sayram_batch_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __len__(self):
        return len(self.problems)

    def step(self, nsteps: int = 1, allow_not_converged: bool = False) -> int:
        allow = (OK, ERR_NOT_CONVERGED) if allow_not_converged else (OK,)
        return check(self._L.sayram_batch_step(self.h, int(nsteps)), "sayram_batch_step", allow)

    def step_host(self, nsteps: int, f_in_ptr: Optional[int], f_out_ptr: Optional[int], allow_not_converged=False) -> int:
        allow = (OK, ERR_NOT_CONVERGED) if allow_not_converged else (OK,)
        return check(self._L.sayram_batch_step_host(self.h, int(nsteps), f_in_ptr, f_out_ptr), "sayram_batch_step_host", allow)

    def f(self, idx: int) -> np.ndarray:
        nx, ny = self.shapes[idx]
        out = np.empty((nx, ny))
        check(self._L.sayram_batch_get_f(self.h, idx, _ptr(out)), "sayram_batch_get_f")
        return out

    def set_f(self, idx: int, f) -> None:
        a = _f64(f)
        check(self._L.sayram_batch_set_f(self.h, idx, _ptr(a)), "sayram_batch_set_f")

    def set_dirichlet(self, idx: int, side: int, v) -> None:
        a = _f64(v)
        check(self._L.sayram_batch_set_dirichlet(self.h, idx, side, _ptr(a), a.size), "sayram_batch_set_dirichlet")

    def set_coeffs(self, idx: int, G, Dxx, Dxy, Dyy, inv_tau) -> None:
        arrs = [_f64(a) for a in (G, Dxx, Dxy, Dyy, inv_tau)]
        check(self._L.sayram_batch_set_coeffs(self.h, idx, *[_ptr(a) for a in arrs]), "sayram_batch_set_coeffs")

    def stats(self, idx: int) -> dict:
        s = sayram_stats()
        check(self._L.sayram_batch_stats(self.h, idx, ctypes.byref(s)), "sayram_batch_stats")
        return s.as_dict()

    def export_system(self, idx: int):
        """(M5, R) assembled from the current f of instance idx, reference (unscaled) form."""
        nx, ny = self.shapes[idx]
        M5 = np.empty((5, nx * ny))
        R = np.empty(nx * ny)
        check(self._L.sayram_batch_export_system(self.h, idx, _ptr(M5), _ptr(R)), "sayram_batch_export_system")
        return M5, R

    def device_bytes(self) -> int:
        return int(self._L.sayram_batch_device_bytes(self.h))

    def stream(self) -> int:
        return int(self._L.sayram_batch_stream(self.h) or 0)

    def record_event(self, slot: int) -> None:
        check(self._L.sayram_batch_record_event(self.h, slot), "sayram_batch_record_event")

    def elapsed_ms(self, slot0: int, slot1: int) -> float:
        ms = ctypes.c_double()
        check(self._L.sayram_batch_elapsed_ms(self.h, slot0, slot1, ctypes.byref(ms)), "sayram_batch_elapsed_ms")
        return ms.value

    def enable_timing(self, on: bool = True) -> None:
        check(self._L.sayram_batch_enable_timing(self.h, 1 if on else 0), "sayram_batch_enable_timing")

    def kernel_times(self) -> dict:
        cap = 64
        names = (ctypes.c_char_p * cap)()
        ms = (ctypes.c_double * cap)()
        cnt = (ctypes.c_longlong * cap)()
        m = self._L.sayram_batch_kernel_times(self.h, names, ms, cnt, cap)
        return {names[k].decode(): (ms[k], cnt[k]) for k in range(min(m, cap))}

    def autotune(self, steps: int = 2):
        """Picks the fastest launch shape on this batch (state restored); returns (chunk, blocks/SM)."""
        ch, gm = ctypes.c_int(), ctypes.c_int()
        check(self._L.sayram_batch_autotune(self.h, int(steps), ctypes.byref(ch), ctypes.byref(gm)), "sayram_batch_autotune")
        return ch.value, gm.value

    def set_dtable(self, idx: int, table) -> None:
        """D fields of instance idx (every instance if idx < 0) interpolated on the device from a
        table with fields alpha0_deg, E, Daa, Dap, Dpp (cases.DTable), as constructD does."""
        keep = [_f64(table.alpha0_deg), _f64(table.E), _f64(table.Daa), _f64(table.Dap), _f64(table.Dpp)]
        na, ne = len(keep[0]), len(keep[1])
        if any(a.shape != (na, ne) for a in keep[2:]):
            raise ValueError("Daa, Dap, Dpp must have shape (len(alpha0_deg), len(E))")
        t = sayram_dtable(na, ne, *[_ptr(a) for a in keep])
        check(self._L.sayram_batch_set_dtable(self.h, int(idx), ctypes.byref(t)), "sayram_batch_set_dtable")

    def set_coop(self, on: bool) -> None:
        """Run each step's refinement loop as one cooperative kernel when the batch's chunks fit in
        one wave of co-resident blocks (default), or always as the loops of separate kernels."""
        check(self._L.sayram_batch_set_coop(self.h, 1 if on else 0), "sayram_batch_set_coop")

    def set_launch_shape(self, chunk: int, blocks_per_sm: int) -> None:
        check(self._L.sayram_batch_set_launch_shape(self.h, int(chunk), int(blocks_per_sm)), "sayram_batch_set_launch_shape")

    def launch_shape(self):
        ch, gm = ctypes.c_int(), ctypes.c_int()
        check(self._L.sayram_batch_get_launch_shape(self.h, ctypes.byref(ch), ctypes.byref(gm)), "sayram_batch_get_launch_shape")
        return ch.value, gm.value

    def tuning_log(self):
        cap = 32
        c, g, m = (ctypes.c_int * cap)(), (ctypes.c_int * cap)(), (ctypes.c_double * cap)()
        n = self._L.sayram_batch_tuning_log(self.h, c, g, m, cap)
        return [{"chunk": c[k], "blocks_per_sm": g[k], "ms_per_step": m[k]} for k in range(min(n, cap))]

    def launches(self) -> int:
        return int(self._L.sayram_batch_launches(self.h))


class Solver(Batch):
    """Drop-in of the reference's ``class Solver`` for one instance (Solver.h:18-26)."""

    def __init__(self, problem, opts: Optional[sayram_options] = None, **kw):
        super().__init__([problem], opts, **kw)
        self.problem = problem

    def update(self) -> None:  # Solver::update, Solver.cc:270-290
        check(self._L.sayram_update(self.h), "sayram_update")

    def t(self) -> float:  # Solver::t, Solver.h:23
        return float(self._L.sayram_t(self.h))

    def f(self, idx: int = 0) -> np.ndarray:  # Solver::f, Solver.h:24
        return super().f(0)

    def set_f(self, f) -> None:  # replaces the state (alpha-major)
        super().set_f(0, f)

    def set_dirichlet(self, side: int, v) -> None:
        super().set_dirichlet(0, side, v)

    def set_coeffs(self, G, Dxx, Dxy, Dyy, inv_tau) -> None:
        super().set_coeffs(0, G, Dxx, Dxy, Dyy, inv_tau)

    def set_dtable(self, table, idx: int = 0) -> None:  # constructD on the device
        super().set_dtable(idx, table)

    def get_stats(self) -> dict:
        return self.stats(0)


class Server:
    """Continuous-batching service of solve requests (sayram_server_*)."""

    def __init__(self, hbm_budget_bytes: float, max_slots: int = 4096, max_side: int = 1024,
                 opts: Optional[sayram_options] = None, lanes: int = 1, split_side: int = 0,
                 small_fraction: float = 0.0, wait_seconds: float = 0.0, **kw):
        L = load()
        self._L = L
        cfg = sayram_server_config(float(hbm_budget_bytes), int(max_slots), int(max_side), int(lanes),
                                   int(split_side), float(small_fraction), float(wait_seconds))
        opts = opts if opts is not None else options(**kw)
        h = ctypes.c_void_p()
        check(L.sayram_server_create(ctypes.byref(cfg), ctypes.byref(opts), ctypes.byref(h)), "sayram_server_create")
        self.h = h
        self.shapes = {}

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            self._L.sayram_server_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, problem, nsteps: int) -> int:
        pack = _Pack([problem])
        rid = ctypes.c_longlong()
        check(self._L.sayram_server_submit(self.h, pack.arr, int(nsteps), ctypes.byref(rid)), "sayram_server_submit")
        self.shapes[rid.value] = (int(problem.nx), int(problem.ny))
        return rid.value

    def tick(self) -> int:
        n = ctypes.c_int()
        check(self._L.sayram_server_tick(self.h, ctypes.byref(n)), "sayram_server_tick")
        return n.value

    def poll(self, rid: int, want_f: bool = True):
        """None while running; else (f or None, stats dict, t_submit, t_done) and the result is released."""
        nx, ny = self.shapes[rid]
        f = np.empty((nx, ny)) if want_f else None
        st = sayram_stats()
        t0, t1 = ctypes.c_double(), ctypes.c_double()
        rc = self._L.sayram_server_poll(self.h, rid, _ptr(f), ctypes.byref(st), ctypes.byref(t0), ctypes.byref(t1))
        if rc == ERR_STATE:
            return None
        check(rc, "sayram_server_poll")
        del self.shapes[rid]
        return f, st.as_dict(), t0.value, t1.value

    def completed_ids(self, cap: int = 4096):
        buf = (ctypes.c_longlong * cap)()
        n = self._L.sayram_server_completed_ids(self.h, buf, cap)
        return [buf[k] for k in range(n)]

    def info(self) -> dict:
        i = sayram_server_info()
        check(self._L.sayram_server_info_get(self.h, ctypes.byref(i)), "sayram_server_info_get")
        return i.as_dict()


def instance_bytes(nx: int, ny: int, precision: int = FP32_REFINE) -> int:
    return int(load().sayram_instance_bytes(nx, ny, precision))


class H5File:
    """The run's HDF5 output file (sayram_h5.h): ``write(path, array)`` is the reference's
    ``xt::dump(file, path, array, xt::dump_mode::overwrite)`` (main.cc:65-89); the file is
    complete after ``close()`` (or the end of a ``with`` block)."""

    def __init__(self, path: str):
        self._L = load()
        self.h = _P()
        check(self._L.sayram_h5_create(os.fsencode(path), ctypes.byref(self.h)), "sayram_h5_create")

    def write(self, path: str, array) -> None:
        if not self.h:
            raise RuntimeError("H5File is closed")
        a = np.require(array, dtype=np.float64, requirements="C")  # keeps 0-d arrays scalars
        dims = (ctypes.c_longlong * max(1, a.ndim))(*a.shape)
        check(self._L.sayram_h5_write(self.h, path.encode(), _ptr(a), a.ndim, dims), "sayram_h5_write")

    def close(self) -> None:
        if self.h:
            h, self.h = self.h, _P()
            check(self._L.sayram_h5_close(h), "sayram_h5_close")

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
        return False

    def __del__(self):  # an unclosed file is finished (and its handle freed) when collected
        try:
            self.close()
        except Exception:
            pass


def h5_read(file: str, path: str) -> np.ndarray:
    """``xt::load_hdf5(file, path)``: one dataset of a classic-format HDF5 file as float64."""
    L = load()
    rank, dims, data = ctypes.c_int(), (ctypes.c_longlong * 32)(), _dp()
    check(L.sayram_h5_read(os.fsencode(file), path.encode(), 32, ctypes.byref(rank), dims, ctypes.byref(data)),
          "sayram_h5_read")
    try:
        shape = tuple(dims[k] for k in range(rank.value))
        n = int(np.prod(shape)) if shape else 1
        return np.ctypeslib.as_array(data, shape=(max(n, 1),))[:n].copy().reshape(shape)
    finally:
        L.sayram_h5_free(ctypes.cast(data, ctypes.c_void_p))


def load_dtable(file: str):
    """``Albert_Young_IO::read_D`` (Albert_Young_IO.cc:17-36): the D table of a D/<dID>.h5 file as
    a cases.DTable (/alpha0 in degrees, /E, /Daa, /Dap, /Dpp)."""
    from .cases import DTable

    L = load()
    t = sayram_dtable()
    check(L.sayram_dtable_load_h5(os.fsencode(file), ctypes.byref(t)), "sayram_dtable_load_h5")
    try:
        na, ne = t.n_alpha, t.n_energy
        vec = lambda p, n: np.ctypeslib.as_array(p, shape=(n,)).copy()
        return DTable(vec(t.alpha0_deg, na), vec(t.energy, ne), vec(t.Daa, na * ne).reshape(na, ne),
                      vec(t.Dap, na * ne).reshape(na, ne), vec(t.Dpp, na * ne).reshape(na, ne))
    finally:
        L.sayram_dtable_free(ctypes.byref(t))
