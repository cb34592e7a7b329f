"""Builds the in-tree native libraries of fsig_gb300.

libfsig.so      the CUDA engine (sm_103a only) behind include/fsig.h
libfsig_gen.so  the host workload generators behind include/fsig_gen.h
FSIG            the command line (csrc/cli.cpp) on libfsig.so

Translation units are compiled in parallel; objects and libraries go to
fsig_gb300/_build/.  A library is rebuilt when any of its sources or headers
is newer than it.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
INCLUDE = ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-Xptxas", "-warn-spills"]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-Wall", "-Wno-unused-function"]
# The generators must give the same graphs on x86-64 and AArch64: no fused
# multiply-add contraction (GCC contracts by default on AArch64).
GEN_FLAGS = ["-ffp-contract=off"]

ENGINE_SOURCES = ["graph_store.cu", "match.cu", "capi.cu", "mpnn.cu", "pcsr.cu", "plan.cu", "reader.cpp"]
GEN_SOURCES = ["gen.cpp"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the fsig_gb300 engine needs the CUDA toolkit to build")


def _newest_input(paths) -> float:
    return max(p.stat().st_mtime for p in paths)


def _deps() -> list[Path]:
    return sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")


def _compile(src: Path, obj: Path, verbose_ptxas: bool) -> None:
    if src.suffix == ".cu":
        flags = list(NVCC_FLAGS) + (["-Xptxas", "-v"] if verbose_ptxas else [])
        _run([_nvcc(), *ARCH, *flags, "-I", str(INCLUDE), "-c", str(src), "-o", str(obj)])
    else:
        _run(["g++", *CXX_FLAGS, "-I", str(INCLUDE), "-I", str(Path(_nvcc()).parent.parent / "include"),
              "-c", str(src), "-o", str(obj)])


def _stale(target: Path, inputs) -> bool:
    return not target.exists() or target.stat().st_mtime < _newest_input(inputs)


def build_engine(force: bool = False, verbose_ptxas: bool = False) -> Path:
    OUT.mkdir(exist_ok=True)
    lib = OUT / "libfsig.so"
    sources = [CSRC / s for s in ENGINE_SOURCES]
    deps = _deps()
    objs = [OUT / (s.name + ".o") for s in sources]
    todo = [(s, o) for s, o in zip(sources, objs) if force or _stale(o, [s, *deps])]
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(todo), os.cpu_count() or 4))) as ex:
        list(ex.map(lambda so: _compile(so[0], so[1], verbose_ptxas), todo))
    if force or todo or _stale(lib, objs):
        _run([_nvcc(), *ARCH, "-shared", "-o", str(lib), *map(str, objs), "-lcudart"])
    return lib


def build_gen(force: bool = False) -> Path:
    OUT.mkdir(exist_ok=True)
    lib = OUT / "libfsig_gen.so"
    sources = [CSRC / s for s in GEN_SOURCES]
    if force or _stale(lib, [*sources, INCLUDE / "fsig_gen.h"]):
        _run(["g++", *CXX_FLAGS, *GEN_FLAGS, "-shared", "-pthread", "-I", str(INCLUDE), "-o", str(lib),
              *map(str, sources)])
    return lib


def build_cli(force: bool = False) -> Path:
    """The FSIG executable, linked against the in-tree libfsig.so."""
    OUT.mkdir(exist_ok=True)
    exe = OUT / "FSIG"
    src = CSRC / "cli.cpp"
    lib = OUT / "libfsig.so"
    if force or _stale(exe, [src, lib, INCLUDE / "fsig.h"]):
        _run(["g++", "-O2", "-std=c++17", "-Wall", "-I", str(INCLUDE), "-o", str(exe), str(src), "-L", str(OUT),
              "-lfsig", "-Wl,-rpath,$ORIGIN"])
    return exe


def build_all(force: bool = False) -> None:
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        futs = [ex.submit(build_engine, force), ex.submit(build_gen, force)]
        for f in futs:
            f.result()
    build_cli(force)


if __name__ == "__main__":
    import sys
    build_all(force="--force" in sys.argv)
    print("built", OUT)
