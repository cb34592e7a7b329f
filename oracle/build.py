"""Build recipe for the CPU oracle (test infrastructure only).

oracle/_build/liboracle.so   the CPU restatement (oracle.cpp), g++ -O2.
oracle/_build/libgen.so      a copy of the workload generators
                             (fsig_gb300/csrc/gen.cpp) for the CPU benchmark
                             arm, which loads no library of the engine.
oracle/_ref/ref_dump         the reference's own CPU sources (reader, graph,
                             format transformer, GSI/MMatch host planning)
                             compiled from the reference tree together with
                             oracle/ref_dump.cc; only when that tree exists.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
REF_OUT = HERE / "_ref"
REFERENCE = Path(os.environ.get("FSIG_REFERENCE_TREE", "/root/reference"))


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"oracle build failed: {' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")


def build_oracle(force: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    lib = BUILD / "liboracle.so"
    srcs = [HERE / "oracle.cpp", HERE / "oracle.h"]
    if force or not lib.exists() or lib.stat().st_mtime < max(s.stat().st_mtime for s in srcs):
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-pthread", "-o", str(lib), str(HERE / "oracle.cpp")])
    return lib


def build_generators(force: bool = False) -> Path:
    """The workload generators, built from the engine's source with the same
    flags (no multiply-add contraction: identical graphs on every platform)."""
    BUILD.mkdir(exist_ok=True)
    lib = BUILD / "libgen.so"
    root = HERE.parent
    srcs = [root / "fsig_gb300" / "csrc" / "gen.cpp", root / "include" / "fsig_gen.h"]
    if force or not lib.exists() or lib.stat().st_mtime < max(s.stat().st_mtime for s in srcs):
        _run(["g++", "-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-shared", "-pthread",
              "-I", str(root / "include"), "-o", str(lib), str(srcs[0])])
    return lib


def build_reference(force: bool = False) -> Path | None:
    """Compiles the reference's CPU-side sources where they lie.

    Shims, all on the command line (the reference tree is read-only):
      -std=c++17                     CCCL in CUDA 13 needs it;
      -DclockRate=major              cudaDeviceProp::clockRate is gone in CUDA 13
                                     (match/subgraph_match.h:67 prints it);
      -gencode compute_103a          the reference Makefile targets sm_75.
    Nothing here runs on a GPU: ref_dump calls host-only methods.
    """
    if not (REFERENCE / "match" / "GSI.cu").exists():
        return None
    REF_OUT.mkdir(exist_ok=True)
    exe = REF_OUT / "ref_dump"
    inputs = [HERE / "ref_dump.cc"]
    if not force and exe.exists() and exe.stat().st_mtime >= max(p.stat().st_mtime for p in inputs):
        return exe
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    r = REFERENCE
    objs = []
    for src in ["graph/graph.cc", "IO/graph_reader.cc", "graph_format_transformer/graph_format_transformer.cc"]:
        obj = REF_OUT / (Path(src).stem + ".o")
        _run(["g++", "-O2", "-std=c++17", "-c", str(r / src), "-o", str(obj)])
        objs.append(obj)
    for src in ["match/GSI.cu", "match/MMatch.cu"]:
        obj = REF_OUT / (Path(src).stem + ".o")
        _run([nvcc, "-std=c++17", "-O2", "-DclockRate=major", "-gencode", "arch=compute_103a,code=sm_103a",
              "-w", "-c", str(r / src), "-o", str(obj)])
        objs.append(obj)
    _run([nvcc, "-std=c++17", "-O2", "-DclockRate=major", "-I", str(r), "-gencode",
          "arch=compute_103a,code=sm_103a", "-w", "-o", str(exe), str(HERE / "ref_dump.cc"), *map(str, objs)])
    return exe


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_generators(force="--force" in sys.argv))
    print(build_reference(force="--force" in sys.argv))
