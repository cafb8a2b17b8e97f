"""Build the oracle (test infrastructure): ``oracle/_build/liboracle.so``.

g++ -std=c++20 -O3 -ffp-contract=off (IEEE-strict: no fast-math, no FMA
contraction, no -march flags so the same code builds on x86-64 and aarch64).
The reference itself needs C++26/GCC 16 and vcpkg dependencies and cannot be
compiled on this toolchain, so there is no oracle/_ref build.
"""

from __future__ import annotations

import os
import pathlib
import subprocess

HERE = pathlib.Path(__file__).resolve().parent
SRC = HERE / "oracle.cpp"
LIB = HERE / "_build" / "liboracle.so"
FLAGS = ["-std=c++20", "-O3", "-ffp-contract=off", "-fno-fast-math", "-fPIC",
         "-shared", "-pthread", "-Wall", "-Wextra", "-Wno-maybe-uninitialized"]


def build(force: bool = False) -> pathlib.Path:
    deps = [SRC, HERE / "oracle.h", HERE.parent / "include" / "titgpu.h", pathlib.Path(__file__)]
    if not force and LIB.exists() and all(d.stat().st_mtime <= LIB.stat().st_mtime for d in deps):
        return LIB
    LIB.parent.mkdir(exist_ok=True)
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [os.environ.get("CXX", "g++"), *FLAGS, "-o", str(tmp), str(SRC)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
