"""include/pt.h compiles as C11 and include/pt_scene.hpp as C++17, and the
Python binding's ctypes structures have the C structures' size and field
offsets (a mismatch would corrupt memory silently).  Host compiler only."""
import ctypes
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include")

STRUCTS = {"pt_options": "Options", "pt_render_params": "RenderParams", "pt_stats": "Stats",
           "pt_batch_item": "BatchItem", "pt_tune": "Tune"}


def test_headers_compile():
    cc, cxx = shutil.which("gcc"), shutil.which("g++")
    if cc is None or cxx is None:
        pytest.skip("no host compiler")
    subprocess.run([cc, "-std=c11", "-Wall", "-Werror", "-fsyntax-only", "-x", "c",
                    os.path.join(INC, "pt.h")], check=True)
    subprocess.run([cxx, "-std=c++17", "-Wall", "-fsyntax-only", "-x", "c++",
                    os.path.join(INC, "pt_scene.hpp")], check=True)


def test_ctypes_layout_matches_c(ptgb_mod, tmp_path):
    cc = shutil.which("gcc")
    if cc is None:
        pytest.skip("no host compiler")
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "pt.h"', "int main(void) {"]
    for cname, pyname in STRUCTS.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for field, _ in getattr(ptgb_mod, pyname)._fields_:
            lines.append(f'  printf("{cname} {field} %zu\\n", offsetof({cname}, {field}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = str(tmp_path / "layout")
    subprocess.run([cc, "-std=c11", "-I", INC, str(src), "-o", exe], check=True)
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {}
    for line in filter(None, out):
        cname, key, value = line.split()
        got[(cname, key)] = int(value)
    for cname, pyname in STRUCTS.items():
        st = getattr(ptgb_mod, pyname)
        assert ctypes.sizeof(st) == got[(cname, "size")], cname
        for field, _ in st._fields_:
            assert getattr(st, field).offset == got[(cname, field)], (cname, field)
