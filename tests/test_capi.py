"""The C-ABI library: builds, loads without a GPU, exports every symbol include/*.h declares, and
rejects bad arguments on the host before touching CUDA. CPU only (no compute calls)."""
import ctypes
import glob
import os
import re

import pytest

from conftest import ROOT


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w\s\*]*?\b(sayram_\w+)\s*\(", src, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_api():
    names = declared_functions()
    for required in ("sayram_create", "sayram_update", "sayram_get_f", "sayram_batch_create",
                     "sayram_batch_step", "sayram_batch_step_host", "sayram_last_error"):
        assert required in names


def test_library_exports_every_declared_symbol(capi):
    lib = ctypes.CDLL(capi.lib_path())
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    # the Python binding covers the whole header
    assert set(declared_functions()) <= set(capi.SIGNATURES)


def test_default_options(capi):
    o = capi.options()
    assert o.precision == capi.FP64 and o.max_iters > 0 and o.max_refine >= 2


def _problem_struct(capi, nx=4, ny=3, bad_edges=False, drop_dirichlet=False):
    from sayram2d_gb300 import cases

    p = cases.synthetic_problem(nx, ny, 1e-2, seed=0)
    if bad_edges:
        p.x_edges = p.x_edges.copy()
        p.x_edges[2] = p.x_edges[1]
    if drop_dirichlet:
        p.dirichlet[0] = None
    return capi._Pack([p])


@pytest.mark.parametrize("kind,needle", [("bad_edges", "strictly increasing"),
                                         ("drop_dirichlet", "Dirichlet BC: missing value")])
def test_invalid_problem_rejected_on_host(capi, kind, needle):
    pack = _problem_struct(capi, **{kind: True})
    h = ctypes.c_void_p()
    rc = capi.load().sayram_batch_create(pack.arr, 1, ctypes.byref(capi.options()), ctypes.byref(h))
    assert rc == capi.ERR_ARG
    assert needle in capi.last_error()
    assert not h.value


def test_null_handles_rejected(capi):
    L = capi.load()
    assert L.sayram_batch_step(None, 1) == capi.ERR_ARG
    assert L.sayram_batch_get_f(None, 0, None) == capi.ERR_ARG
    assert L.sayram_batch_size(None) == 0
    assert L.sayram_batch_autotune(None, 1, None, None) == capi.ERR_ARG
    assert L.sayram_batch_set_dtable(None, 0, None) == capi.ERR_ARG
    assert L.sayram_set_dtable(None, None) == capi.ERR_ARG
    assert L.sayram_batch_set_launch_shape(None, 1024, 8) == capi.ERR_ARG
    assert L.sayram_batch_get_launch_shape(None, None, None) == capi.ERR_ARG


def test_empty_and_bad_requests_rejected_on_host(capi):
    """An empty batch, a negative step count, a null server and a malformed server config are
    refused before any CUDA call."""
    L = capi.load()
    h = ctypes.c_void_p()
    pack = _problem_struct(capi)
    assert L.sayram_batch_create(pack.arr, 0, ctypes.byref(capi.options()), ctypes.byref(h)) == capi.ERR_ARG
    assert "empty batch" in capi.last_error() and not h.value
    assert L.sayram_batch_step_host(None, -1, None, None) == capi.ERR_ARG
    assert L.sayram_server_tick(None, None) == capi.ERR_ARG
    assert L.sayram_server_submit(None, pack.arr, 1, None) == capi.ERR_ARG
    cfg = capi.sayram_server_config(0.0, 4, 64, 1, 0, 0.0)
    assert L.sayram_server_create(ctypes.byref(cfg), ctypes.byref(capi.options()), ctypes.byref(h)) == capi.ERR_ARG
    assert "budget" in capi.last_error()
    assert L.sayram_server_create(None, None, ctypes.byref(h)) == capi.ERR_ARG


def test_instance_bytes_monotone(capi):
    a = capi.instance_bytes(64, 64, capi.FP32_REFINE)
    b = capi.instance_bytes(128, 128, capi.FP32_REFINE)
    c = capi.instance_bytes(128, 128, capi.FP64)
    assert 0 < a < b and c > 0
