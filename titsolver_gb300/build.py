"""Build the in-tree CUDA library ``titsolver_gb300/_lib/libtitgpu.so``.

Every ``csrc/*.cu`` translation unit is compiled for sm_103a in parallel and
linked into one shared library with the C ABI of ``include/titgpu.h``.
``csrc/engine_inst.cu`` is compiled once per engine instance (dimension,
precision form, smoothing kernel: 24 objects), the 3D FP64 instances first,
so that no single object dominates the build time.  Nothing is installed
outside the package directory.
"""

from __future__ import annotations

import concurrent.futures
import os
import pathlib
import shutil
import subprocess
import sys

PKG = pathlib.Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT_DIR = PKG / "_lib"
OBJ_DIR = PKG / "_build"
LIB = OUT_DIR / "libtitgpu.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3",
    "-lineinfo",
    "-std=c++20",
    "--expt-relaxed-constexpr",
    "-Xcompiler",
    "-fPIC",
    "-Xcompiler",
    "-Wall",
    "-Xptxas",
    "-warn-spills",
]


def nvcc() -> str:
    exe = shutil.which("nvcc")
    if exe is None:
        cand = pathlib.Path("/usr/local/cuda/bin/nvcc")
        if cand.exists():
            return str(cand)
        raise RuntimeError("nvcc not found: the CUDA toolkit is required")
    return exe


INSTANCE_SRC = CSRC / "engine_inst.cu"
DIMS = (3, 2)
FORMS = (0, 1)  # TG_FP64, TG_FP32C
KERNELS = range(6)  # TG_KERNEL_*


def _sources() -> list[pathlib.Path]:
    return sorted(CSRC.glob("*.cu"))


def _jobs() -> list[tuple[pathlib.Path, str, list[str]]]:
    """(source, object stem, extra nvcc defines) of every object, the
    slowest first."""
    jobs = [(INSTANCE_SRC, f"engine_{d}d_{'f64' if f == 0 else 'f32'}_k{k}",
             [f"-DTG_INST_DIM={d}", f"-DTG_INST_FORM={f}", f"-DTG_INST_KERNEL={k}"])
            for d in DIMS for f in FORMS for k in KERNELS]
    jobs += [(src, src.stem, []) for src in _sources() if src != INSTANCE_SRC]
    return jobs


def _deps() -> list[pathlib.Path]:
    return sorted(CSRC.glob("*.cuh")) + [ROOT / "include" / "titgpu.h"]


def _compile(job: tuple[pathlib.Path, str, list[str]], verbose: bool) -> pathlib.Path:
    src, stem, defines = job
    obj = OBJ_DIR / (stem + ".o")
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *defines, "-I", str(ROOT / "include"), "-c",
           str(src), "-o", str(obj)]
    if verbose:
        cmd.insert(-4, "-Xptxas=-v")
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed on {stem}:\n{res.stdout}\n{res.stderr}")
    if verbose and res.stderr:
        sys.stderr.write(res.stderr)
    return obj


def up_to_date() -> bool:
    if not LIB.exists():
        return False
    t = LIB.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in _sources() + _deps() + [pathlib.Path(__file__)])


def build(force: bool = False, verbose: bool = False, jobs: int | None = None) -> pathlib.Path:
    """Compile and link the library; returns its path."""
    if not force and up_to_date():
        return LIB
    OUT_DIR.mkdir(exist_ok=True)
    OBJ_DIR.mkdir(exist_ok=True)
    work = _jobs()
    jobs = jobs or min(len(work), max(1, os.cpu_count() or 1))
    for stale in OBJ_DIR.glob("*.o"):
        stale.unlink()
    with concurrent.futures.ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(lambda j: _compile(j, verbose), work))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


HOST_DIR = PKG / "host"
INCLUDE = ROOT / "include"


def build_host(force: bool = False) -> dict[str, pathlib.Path]:
    """Compile the C++ host programs of ``host/*.cpp`` (drivers over the C++
    mirror of ``include/titgpu.hpp``) next to the library; returns name ->
    executable.  Plain g++ for the build machine (no -march flags)."""
    lib = build()
    out = {}
    deps = [lib, *INCLUDE.glob("*.h"), *INCLUDE.glob("*.hpp"), pathlib.Path(__file__)]
    for src in sorted(HOST_DIR.glob("*.cpp")):
        exe = OUT_DIR / src.stem
        fresh = exe.exists() and all(p.stat().st_mtime <= exe.stat().st_mtime
                                     for p in [src, *deps])
        if force or not fresh:
            cmd = [os.environ.get("CXX", "g++"), "-std=c++20", "-O2", "-Wall", "-Wextra",
                   "-I", str(INCLUDE), str(src), "-L", str(OUT_DIR), "-ltitgpu",
                   "-Wl,-rpath,$ORIGIN", "-ldl", "-pthread", "-o", str(exe)]
            res = subprocess.run(cmd, capture_output=True, text=True)
            if res.returncode != 0:
                raise RuntimeError(f"g++ failed on {src.name}:\n{res.stdout}\n{res.stderr}")
        out[src.stem] = exe
    return out


if __name__ == "__main__":
    import argparse

    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--verbose", action="store_true", help="print ptxas register/spill report")
    a = ap.parse_args()
    print(build(force=a.force, verbose=a.verbose))
    for name, exe in build_host(force=a.force).items():
        print(exe)
