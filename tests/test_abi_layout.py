"""The Python binding's ctypes structures have the C header's layout: a C program compiled against
include/sayram_gpu.h prints the size and every field offset of each public struct, and capi's
ctypes.Structure definitions must agree field by field (CPU only)."""
import ctypes
import os
import subprocess

import pytest

from conftest import ROOT

STRUCTS = ["sayram_problem", "sayram_options", "sayram_stats", "sayram_dtable", "sayram_server_config",
           "sayram_server_info"]


def test_ctypes_structs_match_the_header(capi, tmp_path):
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "sayram_gpu.h"', "int main(void) {"]
    for name in STRUCTS:
        cls = getattr(capi, name)
        lines.append(f'  printf("{name} size %zu\\n", sizeof({name}));')
        for field, _ in cls._fields_:
            lines.append(f'  printf("{name}.{field} %zu\\n", offsetof({name}, {field}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    r = subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr  # a field the header lacks fails here
    got = dict(line.rsplit(" ", 1) for line in subprocess.run([str(exe)], capture_output=True, text=True,
                                                               check=True).stdout.splitlines())
    for name in STRUCTS:
        cls = getattr(capi, name)
        assert int(got[f"{name} size"]) == ctypes.sizeof(cls), name
        for field, _ in cls._fields_:
            assert int(got[f"{name}.{field}"]) == getattr(cls, field).offset, (name, field)
