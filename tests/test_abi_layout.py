"""The ctypes mirrors of include/fsig.h's structs have the C compiler's
layout: a C program built from the header prints sizeof and every field's
offsetof, compared with the ctypes structures the Python binding passes
across the boundary.  Needs gcc, no GPU."""
import ctypes as C
import shutil
import subprocess
from pathlib import Path

import pytest

import fsig_gb300 as F

ROOT = Path(__file__).resolve().parent.parent

MIRRORS = {
    "fsig_query": F._Query,
    "fsig_result": F._Result,
    "fsig_batch_opts": F._BatchOpts,
    "fsig_batch_stats": F._Stats,
}


def test_struct_layouts_match_header(tmp_path):
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "fsig.h"', "int main(void) {"]
    for cname, py in MIRRORS.items():
        lines.append(f'  printf("{cname} sizeof %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {}
    for line in filter(None, out):
        cname, field, value = line.split()
        got[(cname, field)] = int(value)
    for cname, py in MIRRORS.items():
        assert got[(cname, "sizeof")] == C.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)
