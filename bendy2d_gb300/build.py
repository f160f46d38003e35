"""Build the bendy2d-gb300 C-ABI library in-tree.

Compiles the CUDA translation unit for sm_103a and the host C++ units in
parallel, then links ``bendy2d_gb300/_build/libbendy2d_gb300.so``.  Float
flags matter for parity with the reference: no FMA contraction anywhere
(``--fmad=false`` on the device, ``-ffp-contract=off`` on the host), IEEE
division and square root, denormals kept.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = BUILD / "libbendy2d_gb300.so"

CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
ARCH = "-gencode=arch=compute_103a,code=sm_103a"

NVCC_FLAGS = [
    ARCH, "-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-prec-div=true",
    "-prec-sqrt=true", "-ftz=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
    "--expt-relaxed-constexpr",
]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-Wall",
             "-Wno-unused-function"]

CU_SOURCES = ["engine.cu", "noalloc.cu"]
CXX_SOURCES = ["host.cpp", "planner.cpp", "capi.cpp", "server.cpp"]
HEADERS = ["b2d_dev.h", "kernels.cuh", "engine.hpp", "host.hpp", "server.hpp"]


def _nvcc() -> str:
    p = CUDA_HOME / "bin" / "nvcc"
    return str(p) if p.exists() else (shutil.which("nvcc") or "nvcc")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps if d.exists())


def build(force: bool = False, verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    inc = ["-I", str(CSRC), "-I", str(PKG.parent / "include"), "-I", str(CUDA_HOME / "include")]
    headers = [CSRC / h for h in HEADERS] + [PKG.parent / "include" / "bendy2d.h"]
    jobs = []
    objs = []
    for src in CU_SOURCES:
        obj = BUILD / (src + ".o")
        objs.append(obj)
        if force or _stale(obj, [CSRC / src] + headers):
            jobs.append([_nvcc(), *NVCC_FLAGS, *inc, "-c", str(CSRC / src), "-o", str(obj)])
    for src in CXX_SOURCES:
        obj = BUILD / (src + ".o")
        objs.append(obj)
        if force or _stale(obj, [CSRC / src] + headers):
            jobs.append(["g++", *CXX_FLAGS, *inc, "-c", str(CSRC / src), "-o", str(obj)])
    if jobs:
        with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            list(ex.map(_run, jobs))
    if force or jobs or _stale(LIB, objs):
        libdir = CUDA_HOME / "lib64"
        tmp = LIB.with_suffix(".so.tmp")
        _run(["g++", "-shared", "-o", str(tmp), *map(str, objs), f"-L{libdir}",
              f"-Wl,-rpath,{libdir}", "-lcudart", "-lpthread"])
        os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
