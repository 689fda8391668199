"""Builds libp3x.so in-tree (CUDA for sm_103a + host C++), in parallel.

Objects go to scream_gb300/_build/, the library to scream_gb300/libp3x.so.
A translation unit is recompiled when any source or header is newer than its
object.  Run ``python -m scream_gb300.build`` or call :func:`build`.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
BUILD = PKG / "_build"
LIB = PKG / "libp3x.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FP32_BULK_FLAGS = ["--use_fast_math", "-ftz=false"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the P3 CUDA library cannot be built")


def _deps_mtime() -> float:
    files = list(CSRC.glob("*")) + list(INCLUDE.glob("*.h")) + [Path(__file__)]
    return max(f.stat().st_mtime for f in files)


def _compile(src: Path, newest: float) -> Path:
    obj = BUILD / (src.name + ".o")
    if obj.exists() and obj.stat().st_mtime >= newest:
        return obj
    nvcc = _nvcc()
    if src.suffix == ".cu":
        cmd = [nvcc, "-std=c++17", "-O3", *ARCH, "-lineinfo", "-Xcompiler", "-fPIC,-fopenmp",
               f"-I{INCLUDE}", f"-I{CSRC}", "-c", str(src), "-o", str(obj)]
        if src.name.startswith("p3x_k_f"):
            # FP32-bulk kernels: FP32 rates through the hardware approximations
            # (approximate division, square root and transcendentals); FP64
            # arithmetic is unaffected, denormals are kept, and the exact
            # building blocks (double-float sums, table indices) use
            # correctly rounded intrinsics.
            cmd[3:3] = FP32_BULK_FLAGS
    else:
        cmd = ["g++", "-std=c++17", "-O3", "-fPIC", "-fopenmp", f"-I{INCLUDE}", f"-I{CSRC}",
               "-I/usr/local/cuda/include", "-c", str(src), "-o", str(obj)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    return obj


def build(jobs: int | None = None, verbose: bool = False) -> Path:
    """Compiles every CUDA and C++ source of libp3x and links the shared library."""
    BUILD.mkdir(exist_ok=True)
    srcs = sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))
    newest = _deps_mtime()
    jobs = jobs or max(2, os.cpu_count() or 2)
    # the largest translation units first
    srcs.sort(key=lambda p: (not p.name.startswith("p3x_k_"), p.name))
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, newest), srcs))
    if LIB.exists() and LIB.stat().st_mtime >= max(o.stat().st_mtime for o in objs):
        return LIB
    cmd = [_nvcc(), "-shared", *ARCH, "-o", str(LIB), *map(str, objs), "-Xcompiler", "-fopenmp", "-lgomp"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
