"""The ctypes mirrors of include/fsig.h's structs have the C compiler's
layout: a C program built from the header prints sizeof and every field's
offsetof, compared with the ctypes structures the Python binding passes
across the boundary; the binding's constants have the header's values.
Needs gcc, no GPU."""
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


CONSTANTS = {
    "FSIG_OK": F.OK, "FSIG_EINVAL": F.EINVAL, "FSIG_ENODEV": F.ENODEV, "FSIG_ECUDA": F.ECUDA,
    "FSIG_EADMISSION": F.EADMISSION, "FSIG_ENOGRAPH": F.ENOGRAPH, "FSIG_EQUERY": F.EQUERY, "FSIG_EIO": F.EIO,
    "FSIG_ETIMEOUT": F.ETIMEOUT, "FSIG_EOVERFLOW": F.EOVERFLOW, "FSIG_ELIMIT": F.ELIMIT,
    "FSIG_ALGO_FSIG": F.ALGO_FSIG, "FSIG_ALGO_GSI": F.ALGO_GSI, "FSIG_ALGO_FUSED": F.ALGO_FUSED,
    "FSIG_ORDER_HEURISTIC": F.ORDER_HEURISTIC, "FSIG_ORDER_LEARNED": F.ORDER_LEARNED,
    "FSIG_ORDER_GIVEN": F.ORDER_GIVEN, "FSIG_SEGMENTS_AUTO": F.SEGMENTS_AUTO,
    "FSIG_SEGMENTS_TABLE": F.SEGMENTS_TABLE, "FSIG_SEGMENTS_ROWS": F.SEGMENTS_ROWS,
    "FSIG_MAX_QUERY": F.MAX_QUERY, "FSIG_HASH_SEED": F.HASH_SEED,
}


def test_constants_match_header(tmp_path):
    """Every status, algorithm, order and segment-index constant the binding
    passes has the header's value."""
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    lines = ["#include <stdio.h>", '#include "fsig.h"', "int main(void) {"]
    lines += [f'  printf("{name} %lld\\n", (long long){name});' for name in CONSTANTS]
    lines += ["  return 0;", "}"]
    src = tmp_path / "consts.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "consts"
    subprocess.run(["gcc", "-std=c11", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {name: int(v) for name, v in (line.split() for line in out if line)}
    for name, want in CONSTANTS.items():
        assert got[name] % (1 << 64) == want % (1 << 64), name
