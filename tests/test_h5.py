"""The HDF5 output writer (include/sayram_h5.h) and the main.cc loop that uses it (run.py).

The writer is host code: everything here but the last test runs without a GPU. Its files are
read back with tests/h5read.py, a strict reader of the classic HDF5 format that is itself pinned
against a file written by libhdf5 (scipy's MATLAB 7.3 test file, when scipy ships it) and
against scipy's reading of the same variable from a MATLAB 5 file.
"""
import os
import struct

import numpy as np
import pytest

import h5read
from conftest import ROOT

SCIPY_MAT = None
try:
    import scipy.io

    SCIPY_MAT = os.path.join(os.path.dirname(scipy.io.__file__), "matlab", "tests", "data")
except ImportError:  # pragma: no cover
    pass

LIBHDF5_FILE = os.path.join(SCIPY_MAT, "testhdf5_7.4_GLNX86.mat") if SCIPY_MAT else ""
MAT5_FILE = os.path.join(SCIPY_MAT, "testdouble_7.4_GLNX86.mat") if SCIPY_MAT else ""
needs_libhdf5_file = pytest.mark.skipif(not os.path.exists(LIBHDF5_FILE),
                                        reason="scipy's libhdf5-written test file is not installed")


# ----------------------------------------------------------------------------- the reader
@needs_libhdf5_file
def test_reader_reads_a_libhdf5_file():
    f = h5read.File(LIBHDF5_FILE)
    assert f.base == 512  # MATLAB's user block
    ds = f["/testdouble"]
    assert ds.dtype == np.float64 and ds.layout == "contiguous" and ds.shape == (9, 1)
    assert ds.attributes == ["MATLAB_class"]
    if os.path.exists(MAT5_FILE):
        ref = scipy.io.loadmat(MAT5_FILE)["testdouble"]  # the same variable, MATLAB 5 format
        np.testing.assert_array_equal(ds.data.ravel(), ref.ravel())


@needs_libhdf5_file
def test_reader_rejects_a_damaged_file(tmp_path):
    buf = bytearray(open(LIBHDF5_FILE, "rb").read())
    i = buf.find(b"SNOD")
    buf[i:i + 4] = b"SNOX"
    p = tmp_path / "bad.h5"
    p.write_bytes(bytes(buf))
    with pytest.raises(h5read.H5FormatError):
        h5read.File(str(p))


# ----------------------------------------------------------------------------- the writer
def _write(capi, path, items):
    with capi.H5File(str(path)) as h5:
        for name, arr in items:
            h5.write(name, arr)


def test_round_trip_of_the_reference_layout(capi, tmp_path):
    rng = np.random.default_rng(3)
    nx, ny, nplots = 9, 7, 12
    alpha0 = np.linspace(5, 90, nx)
    logEN = rng.standard_normal(ny)
    fs = [rng.standard_normal((nx, ny)) for _ in range(nplots + 1)]
    items = [("/alpha0", alpha0), ("/logEN", logEN)] + [(f"/f/{k}", fs[k]) for k in range(nplots + 1)]
    items.append(("/t", np.linspace(0, 1, nplots + 1)))
    p = tmp_path / "out.h5"
    _write(capi, p, items)
    f = h5read.File(str(p))
    assert f.eof == os.path.getsize(p)
    assert sorted(f.root.members) == ["alpha0", "f", "logEN", "t"]
    # names in the group's byte order, as the B-tree's comparison wants
    assert list(f["/f"].members) == sorted(str(k) for k in range(nplots + 1))
    for name, arr in items:
        ds = f[name]
        assert ds.shape == arr.shape and ds.dtype == np.dtype("<f8")
        np.testing.assert_array_equal(ds.data, arr)


def test_overwrite_scalars_empty_and_nesting(capi, tmp_path):
    p = tmp_path / "misc.h5"
    _write(capi, p, [("/a/b/c", np.arange(6.0).reshape(2, 3)), ("/a/b/c", np.ones(4)), ("/s", np.array(2.5)),
                     ("/e", np.zeros((0, 3))), ("x", np.array([np.inf, -0.0, np.nan, 5e-324]))])
    f = h5read.File(str(p))
    np.testing.assert_array_equal(f["/a/b/c"].data, np.ones(4))  # dump_mode::overwrite
    assert f["/s"].shape == () and float(f["/s"].data) == 2.5
    assert f["/e"].shape == (0, 3) and f["/e"].address == h5read.UNDEF
    x = f["/x"].data
    assert np.isinf(x[0]) and np.signbit(x[1]) and np.isnan(x[2]) and x[3] == 5e-324


def test_many_entries_in_one_group(capi, tmp_path):
    p = tmp_path / "many.h5"
    n = 1001
    _write(capi, p, [(f"/f/{k}", np.full(3, float(k))) for k in range(n)])
    f = h5read.File(str(p))
    assert f.leaf_k >= (n + 1) // 2
    assert len(f["/f"].members) == n
    for k in (0, 7, 500, 1000):
        np.testing.assert_array_equal(f[f"/f/{k}"].data, np.full(3, float(k)))


@needs_libhdf5_file
def test_message_encodings_match_libhdf5(capi, tmp_path):
    """The datatype and fill-value messages of a float64 dataset are byte for byte the ones
    libhdf5 wrote for the float64 dataset of its own file."""
    ref = h5read.File(LIBHDF5_FILE)
    p = tmp_path / "one.h5"
    _write(capi, p, [("/testdouble", np.zeros((9, 1)))])
    ours = h5read.File(str(p))

    def msgs(f):
        stab = f._messages(f.root_ohdr)[0]
        bt, hp = struct.unpack_from("<QQ", stab.body)
        heap, _ = f._heap(hp)
        snod = f._abs(f._btree_leaves(bt, heap)[0])
        _n, oaddr, _c, _r = struct.unpack_from("<QQII", f.buf, snod + 8)
        return {m.type: m for m in f._messages(oaddr)}

    a, b = msgs(ref), msgs(ours)
    for t in (0x3, 0x5):
        assert a[t].body == b[t].body and a[t].flags == b[t].flags
    assert a[0x1].body == b[0x1].body  # dataspace version 1, (9, 1)
    # superblock fields other than addresses
    assert ours.leaf_k == ref.leaf_k and ours.internal_k == ref.internal_k


@pytest.mark.parametrize("name,arr,needle", [
    ("/a", np.ones(2), "is a dataset"),  # then /a/b below
    ("/", np.ones(2), "empty dataset name"),
    ("/x/../y", np.ones(2), "'.' or '..'"),
])
def test_bad_paths_rejected(capi, tmp_path, name, arr, needle):
    h5 = capi.H5File(str(tmp_path / "bad.h5"))
    try:
        if needle == "is a dataset":
            h5.write(name, arr)
            name = "/a/b"
        with pytest.raises(RuntimeError, match=needle):
            h5.write(name, arr)
    finally:
        h5.close()


def test_group_path_cannot_become_a_dataset(capi, tmp_path):
    with capi.H5File(str(tmp_path / "g.h5")) as h5:
        h5.write("/f/0", np.ones(2))
        with pytest.raises(RuntimeError, match="is a group"):
            h5.write("/f", np.ones(2))


def test_null_and_io_errors(capi, tmp_path):
    import ctypes

    L = capi.load()
    assert L.sayram_h5_close(None) == capi.ERR_ARG
    assert L.sayram_h5_write(None, b"/a", None, 0, None) == capi.ERR_ARG
    h = ctypes.c_void_p()
    assert L.sayram_h5_create(str(tmp_path / "no" / "such" / "dir.h5").encode(), ctypes.byref(h)) == capi.ERR_IO
    assert "cannot create" in capi.last_error()


CPP_PROGRAM = r'''
#include <array>
#include <cstdio>
#include "H5File.h"
struct Grid2 {  // an xtensor-like (nx, ny) array: data() and shape()
  std::array<std::size_t, 2> s{3, 2};
  double d[6] = {1, 2, 3, 4, 5, 6};
  const std::array<std::size_t, 2>& shape() const { return s; }
  const double* data() const { return d; }
};
int main(int, char** argv) {
  sayram::H5File file(argv[1]);
  Grid2 f;
  file.dump("/f/0", f);
  const double a[3] = {5.0, 47.5, 90.0};
  file.dump("/alpha0", a, {3});
  try {
    file.dump("/f", a, {3});
  } catch (const std::runtime_error& e) {
    std::printf("%s\n", e.what());
  }
  file.close();
  return 0;
}
'''


def test_cpp_wrapper_writes_the_file(capi, tmp_path):
    """host/H5File.h, the replacement of main.cc's HighFive/xt::dump lines, from C++."""
    import subprocess

    src = tmp_path / "h5main.cc"
    src.write_text(CPP_PROGRAM)
    exe = tmp_path / "h5main"
    libdir = os.path.dirname(capi.lib_path())
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "sayram-2d_gb300", "host"),
                    "-I", os.path.join(ROOT, "include"), str(src), "-L", libdir, "-lsayram_gpu",
                    f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    out = subprocess.run([str(exe), str(tmp_path / "cc.h5")], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "sayram_h5_write" in out.stdout and "is a group" in out.stdout
    f = h5read.File(str(tmp_path / "cc.h5"))
    np.testing.assert_array_equal(f["/f/0"].data, np.arange(1.0, 7.0).reshape(3, 2))
    np.testing.assert_array_equal(f["/alpha0"].data, [5.0, 47.5, 90.0])


# ----------------------------------------------------------------------------- the reader in the library
@needs_libhdf5_file
def test_library_reader_reads_a_libhdf5_file(capi):
    """sayram_h5_read on a file libhdf5 wrote (with a 512-byte user block), against scipy's
    reading of the same variable from its MATLAB 5 copy."""
    d = capi.h5_read(LIBHDF5_FILE, "/testdouble")
    assert d.shape == (9, 1)
    if os.path.exists(MAT5_FILE):
        np.testing.assert_array_equal(d.ravel(), scipy.io.loadmat(MAT5_FILE)["testdouble"].ravel())
    with pytest.raises(RuntimeError, match="no object named"):
        capi.h5_read(LIBHDF5_FILE, "/nothing")


def test_library_reader_round_trip(capi, tmp_path):
    rng = np.random.default_rng(11)
    items = {"/a": rng.standard_normal((4, 5)), "/g/h/b": rng.standard_normal(7), "/s": np.array(1.25),
             "/e": np.zeros((0, 2))}
    items.update({f"/f/{k}": rng.standard_normal((3, 2)) for k in range(40)})
    p = tmp_path / "rt.h5"
    _write(capi, p, list(items.items()))
    for name, arr in items.items():
        got = capi.h5_read(str(p), name)
        assert got.shape == arr.shape
        np.testing.assert_array_equal(got, arr)
    with pytest.raises(RuntimeError, match="is a group"):
        capi.h5_read(str(p), "/g/h")
    with pytest.raises(RuntimeError, match="cannot open"):
        capi.h5_read(str(tmp_path / "missing.h5"), "/a")


def _patched(src, dst, old: bytes, new: bytes):
    buf = open(src, "rb").read()
    assert buf.count(old) == 1
    open(dst, "wb").write(buf.replace(old, new))


def test_library_reader_refuses_what_it_does_not_read(capi, tmp_path):
    p = tmp_path / "x.h5"
    _write(capi, p, [("/a", np.arange(4.0))])
    ds = h5read.File(str(p))["/a"]
    lay = b"\x03\x01" + struct.pack("<QQ", ds.address, ds.size)
    _patched(p, tmp_path / "chunked.h5", lay, b"\x03\x02" + lay[2:])  # layout class 2: chunked
    with pytest.raises(RuntimeError, match="chunked storage"):
        capi.h5_read(str(tmp_path / "chunked.h5"), "/a")
    sig = b"\x89HDF\r\n\x1a\n\x00"
    _patched(p, tmp_path / "v2.h5", sig, sig[:-1] + b"\x02")  # superblock version 2
    with pytest.raises(RuntimeError, match="superblock version 2"):
        capi.h5_read(str(tmp_path / "v2.h5"), "/a")
    (tmp_path / "not.h5").write_bytes(b"plain text, not HDF5" * 40)
    with pytest.raises(RuntimeError, match="not an HDF5 file"):
        capi.h5_read(str(tmp_path / "not.h5"), "/a")


F64_TYPE = bytes.fromhex("11203f00" "08000000" "00004000340b0034ff030000")  # IEEE binary64 LE
F32_TYPE = bytes.fromhex("11201f00" "04000000" "0000200017080017" "7f000000")  # IEEE binary32 LE


def test_library_reader_binary32_and_big_endian(capi, tmp_path):
    """Files whose datasets are binary32 or big-endian (as other writers produce): the same raw
    bytes under a patched datatype message read back as what those bytes mean."""
    a = np.random.default_rng(5).standard_normal(6)
    p = tmp_path / "a.h5"
    _write(capi, p, [("/a", a)])
    # binary32: the 48 bytes of six doubles are twelve floats
    space6 = b"\x01\x01\x00\x00\x00\x00\x00\x00" + struct.pack("<Q", 6)
    buf = open(p, "rb").read()
    assert buf.count(F64_TYPE) == 1 and buf.count(space6) == 1
    f32 = buf.replace(F64_TYPE, F32_TYPE).replace(space6, space6[:8] + struct.pack("<Q", 12))
    (tmp_path / "f32.h5").write_bytes(f32)
    got = capi.h5_read(str(tmp_path / "f32.h5"), "/a")
    np.testing.assert_array_equal(got, np.frombuffer(a.tobytes(), dtype="<f4").astype(np.float64))
    # big-endian binary64: byte-swapped data under the byte-order bit
    q = tmp_path / "b.h5"
    _write(capi, q, [("/a", a.byteswap())])
    be = F64_TYPE[:1] + bytes([F64_TYPE[1] | 1]) + F64_TYPE[2:]
    (tmp_path / "be.h5").write_bytes(open(q, "rb").read().replace(F64_TYPE, be))
    np.testing.assert_array_equal(capi.h5_read(str(tmp_path / "be.h5"), "/a"), a)


def test_library_reader_refuses_absurd_dimensions(capi, tmp_path):
    p = tmp_path / "a.h5"
    _write(capi, p, [("/a", np.arange(4.0))])
    space4 = b"\x01\x01\x00\x00\x00\x00\x00\x00" + struct.pack("<Q", 4)
    _patched(p, tmp_path / "huge.h5", space4, space4[:8] + struct.pack("<Q", 1 << 50))
    with pytest.raises(RuntimeError, match="out of range|differs|larger than its file"):
        capi.h5_read(str(tmp_path / "huge.h5"), "/a")


def test_load_dtable(capi, tmp_path):
    """Albert_Young_IO::read_D: a D file written in the reference's layout loads bit for bit;
    mismatched shapes and missing datasets are refused."""
    from sayram2d_gb300 import cases

    t = cases.synthetic_dtable(5)
    p = tmp_path / "D.h5"
    _write(capi, p, [("/alpha0", t.alpha0_deg), ("/E", t.E), ("/Daa", t.Daa), ("/Dap", t.Dap), ("/Dpp", t.Dpp)])
    u = capi.load_dtable(str(p))
    for k in ("alpha0_deg", "E", "Daa", "Dap", "Dpp"):
        np.testing.assert_array_equal(getattr(u, k), getattr(t, k))
    bad = tmp_path / "Dbad.h5"
    _write(capi, bad, [("/alpha0", t.alpha0_deg), ("/E", t.E), ("/Daa", t.Daa.T), ("/Dap", t.Dap), ("/Dpp", t.Dpp)])
    with pytest.raises(RuntimeError, match="must be \\(n_alpha0, n_E\\)"):
        capi.load_dtable(str(bad))
    missing = tmp_path / "Dmiss.h5"
    _write(capi, missing, [("/alpha0", t.alpha0_deg), ("/E", t.E)])
    with pytest.raises(RuntimeError, match="no object named 'Daa'"):
        capi.load_dtable(str(missing))


C_PROGRAM = r'''
#include <stdio.h>
#include "sayram_h5.h"
int main(int argc, char** argv) {
  (void)argc;
  double a[3] = {5.0, 47.5, 90.0}, f[6] = {1, 2, 3, 4, 5, 6};
  long long d1[1] = {3}, d2[2] = {3, 2};
  sayram_h5 h;
  if (sayram_h5_create(argv[1], &h) != SAYRAM_OK) return 1;
  if (sayram_h5_write(h, "/alpha0", a, 1, d1) != SAYRAM_OK) return 2;
  if (sayram_h5_write(h, "/f/0", f, 2, d2) != SAYRAM_OK) return 3;
  if (sayram_h5_close(h) != SAYRAM_OK) return 4;
  double* back = NULL;
  int rank = 0;
  long long dims[4];
  if (sayram_h5_read(argv[1], "/f/0", 4, &rank, dims, &back) != SAYRAM_OK) return 5;
  printf("%d %lld %lld %g\n", rank, dims[0], dims[1], back[5]);
  sayram_h5_free(back);
  sayram_dtable t;
  if (sayram_dtable_load_h5(argv[1], &t) == SAYRAM_OK) return 6;  /* no /E: refused */
  printf("%s\n", sayram_last_error());
  return 0;
}
'''


def test_c_callers(capi, tmp_path):
    """include/sayram_h5.h from C (C99): write, read back, and a refused D-table load."""
    import subprocess

    src = tmp_path / "h5.c"
    src.write_text(C_PROGRAM)
    exe = tmp_path / "h5c"
    libdir = os.path.dirname(capi.lib_path())
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-L", libdir, "-lsayram_gpu",
                    f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    out = subprocess.run([str(exe), str(tmp_path / "c.h5")], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, (out.returncode, out.stdout, out.stderr)
    first, second = out.stdout.strip().splitlines()
    assert first == "2 3 2 6"
    assert "no object named 'E'" in second
    assert h5read.File(str(tmp_path / "c.h5"))["/alpha0"].data.tolist() == [5.0, 47.5, 90.0]


# ----------------------------------------------------------------------------- the main.cc loop
def test_run_main_takes_at_most_one_argument(capsys):
    from sayram2d_gb300 import run

    assert run.main(["a.ini", "b.ini"]) == 1
    assert "at most one argument" in capsys.readouterr().err


def test_run_rejects_a_mismatched_problem(capi, tmp_path):
    from sayram2d_gb300 import cases, run

    ini = os.path.join(ROOT, "sayram-2d_gb300", "configs", "c0.ini")
    with pytest.raises(ValueError, match="differs"):
        run.run(ini, root=str(tmp_path), problem=cases.synthetic_problem(8, 8, 1e-3, 0))
    with pytest.raises(ValueError, match="precision"):
        run.run(ini, root=str(tmp_path), precision="fp16")


@pytest.mark.gpu
def test_run_writes_what_the_solver_computes(capi, tmp_path):
    """main.cc's loop end to end on a short c0 run: the file holds the axes, f after every
    save_every_step steps (bit-identical to stepping a Solver directly) and t."""
    import math

    from sayram2d_gb300 import cases, run

    ini = tmp_path / "short.ini"
    src = open(os.path.join(ROOT, "sayram-2d_gb300", "configs", "c0.ini")).read()
    ini.write_text(src.replace("nsteps = 1000", "nsteps = 25").replace("nplots = 10", "nplots = 4"))
    rp = cases.read_ini(str(ini))
    assert (rp.nsteps, rp.save_every_step) == (24, 6)  # Parameters.cc:58-60 rounding
    path = run.run(str(ini), root=str(tmp_path))
    assert path == str(tmp_path / "output" / rp.run_id / (rp.run_id + "_data.h5"))
    assert (tmp_path / "output" / rp.run_id / (rp.run_id + ".ini")).read_text() == ini.read_text()
    f = h5read.File(path)
    prob = cases.problem_from_params(rp)
    x = 0.5 * (prob.x_edges[:-1] + prob.x_edges[1:])
    y = 0.5 * (prob.y_edges[:-1] + prob.y_edges[1:])
    np.testing.assert_array_equal(f["/alpha0"].data, x / cases.PI * 180.0)
    np.testing.assert_array_equal(f["/logEN"].data, y - math.log(cases.E0))
    np.testing.assert_array_equal(f["/t"].data, np.linspace(0.0, rp.T, rp.nplots + 1))
    s = capi.Solver(prob, precision=capi.FP64, tol=rp.tol)
    try:
        np.testing.assert_array_equal(f["/f/0"].data, prob.f0)
        for k in range(1, rp.nplots + 1):
            for _ in range(rp.save_every_step):
                s.update()
            np.testing.assert_array_equal(f[f"/f/{k}"].data, s.f())
    finally:
        s.close()
    assert sorted(f["/f"].members, key=int) == [str(k) for k in range(rp.nplots + 1)]
