"""Builds the native library ``librlic_gb300.so`` in-tree with nvcc (sm_103a).

The library is plain CUDA C++ with a C ABI (``include/rlic_gb300.h``); Python
loads it with ctypes, so no torch extension machinery is involved.  Each
translation unit compiles in parallel, then one link step produces the shared
object next to this file.

Floating-point flags matter for parity with the reference: ``-fmad=false``
keeps the compiler from contracting products and sums that the reference
rounds separately, ``-prec-div=true`` keeps divisions IEEE round-to-nearest
and ``-ftz=false`` keeps subnormals.  The device code also spells every
rounding out with ``__*_rn`` intrinsics, so the flags are a second guard.
"""

from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
REPO_DIR = PKG_DIR.parent
CSRC = PKG_DIR / "csrc"
BUILD_DIR = PKG_DIR / "_build"
LIB_NAME = "librlic_gb300.so"
LIB_PATH = PKG_DIR / LIB_NAME

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3",
    "-std=c++17",
    "-lineinfo",
    "-fmad=false",
    "-prec-div=true",
    "-prec-sqrt=true",
    "-ftz=false",
    "-Xcompiler",
    "-fPIC,-O2,-fvisibility=hidden",
    "-Xptxas",
    "-warn-spills",
]

SOURCES = [
    "lic_capi.cu",
    "lic_kernels_f32.cu",
    "lic_kernels_f64.cu",
    "lic_lowp.cu",
    "lic_batch.cu",
    "lic_equalize.cu",
    "lic_stage.cu",
]


def nvcc_path() -> str:
    cand = shutil.which("nvcc")
    if cand:
        return cand
    cuda_home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    path = Path(cuda_home) / "bin" / "nvcc"
    if path.exists():
        return str(path)
    raise RuntimeError("nvcc not found: set CUDA_HOME or put nvcc on PATH")


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> Path:
    """Compile every CUDA translation unit and link ``librlic_gb300.so``."""
    nvcc = nvcc_path()
    BUILD_DIR.mkdir(exist_ok=True)
    headers = sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + [
        REPO_DIR / "include" / "rlic_gb300.h"
    ]
    objs: list[Path] = []
    jobs: list[list[str]] = []
    for src in SOURCES:
        src_path = CSRC / src
        obj = BUILD_DIR / (Path(src).stem + ".o")
        objs.append(obj)
        if force or _stale(obj, [src_path, *headers]):
            jobs.append(
                [nvcc, *ARCH_FLAGS, *NVCC_FLAGS, "-c", str(src_path), "-o", str(obj)]
            )

    def run(cmd: list[str]) -> None:
        if verbose:
            print(" ".join(cmd), flush=True)
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(
                f"nvcc failed ({res.returncode}):\n{' '.join(cmd)}\n{res.stdout}\n{res.stderr}"
            )
        if verbose and (res.stdout or res.stderr):
            print(res.stdout + res.stderr, flush=True)

    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 1)) as ex:
            list(ex.map(run, jobs))
    if force or jobs or _stale(LIB_PATH, objs):
        run(
            [
                nvcc,
                *ARCH_FLAGS,
                "-shared",
                "-o",
                str(LIB_PATH),
                *map(str, objs),
                "-lcudart_static",
                "-lrt",
                "-ldl",
                "-lpthread",
            ]
        )
    return LIB_PATH


if __name__ == "__main__":
    print(build(verbose=True))
