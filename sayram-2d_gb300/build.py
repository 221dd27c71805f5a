"""Builds the CUDA shared library (sm_103a) in-tree: ``_build/libsayram_gpu.so``."""
from __future__ import annotations

import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT_DIR = os.path.join(PKG, "_build")
LIB = os.path.join(OUT_DIR, "libsayram_gpu.so")
SOURCES = ["sayram_engine.cu", "h5_writer.cc", "h5_reader.cc"]
DEPS = ["sayram_kernels.cuh", "sayram_ops.cuh", "dword.cuh", "host_errors.h"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libsayram_gpu.so")


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    files = [os.path.join(CSRC, f) for f in SOURCES + DEPS] + [
        os.path.join(ROOT, "include", h) for h in ("sayram_gpu.h", "sayram_h5.h")]
    return any(os.path.getmtime(f) > t for f in files)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compiles csrc/*.cu with nvcc for sm_103a into _build/libsayram_gpu.so (if stale)."""
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + ".tmp"
    # host code: no fused multiply-adds, so host-side values (grid weights, D-table row factors)
    # are the same separately rounded operations on x86-64 and aarch64
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", "-shared",
           "-I", os.path.join(ROOT, "include"), "-o", tmp] + [os.path.join(CSRC, s) for s in SOURCES]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB
