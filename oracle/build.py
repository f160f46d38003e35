"""Build recipe for the CPU oracle (test infrastructure only).

Compiles oracle/b2d_oracle.c into oracle/_build/libb2d_oracle.so with
-ffp-contract=off (rustc never fuses multiply-add) and no fast-math.  The
reference crate itself is Rust and cannot be compiled here (no Rust
toolchain), so there is no oracle/_ref build.
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "libb2d_oracle.so"
FLAGS = ["-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
         "-fno-unsafe-math-optimizations", "-Wall"]


def build(force: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    src = HERE / "b2d_oracle.c"
    hdr = HERE / "b2d_oracle.h"
    if (force or not LIB.exists() or LIB.stat().st_mtime < max(src.stat().st_mtime,
                                                                 hdr.stat().st_mtime)):
        tmp = LIB.with_suffix(".so.tmp")
        r = subprocess.run(["gcc", *FLAGS, str(src), "-o", str(tmp), "-lm"],
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + r.stderr)
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
