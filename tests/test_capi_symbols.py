"""The C-ABI libraries load without a GPU and export every function their
headers in include/ declare."""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared(header):
    text = (ROOT / "include" / header).read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(fsig_\w+)\s*\(", text)))


@pytest.mark.parametrize("header,lib", [("fsig.h", "libfsig.so"), ("fsig_gen.h", "libfsig_gen.so")])
def test_exports(header, lib):
    path = ROOT / "fsig_gb300" / "_build" / lib
    if not path.exists():
        from fsig_gb300 import _build
        _build.build_all()
    so = ctypes.CDLL(str(path))
    names = declared(header)
    assert len(names) >= 7
    missing = [n for n in names if not hasattr(so, n)]
    assert not missing, missing


def test_engine_refuses_without_gpu_or_loads_with_one():
    import fsig_gb300 as F
    L = F.engine_library()
    assert L.fsig_status_string(F.EADMISSION).decode().startswith("request")
