"""Build recipe of the kinfu_gb300 shared library (sm_103a only).

Compiles the CUDA translation units under ``csrc/`` in parallel with nvcc and links
them into ``kinect_fusion_slam_gb300/lib/libkinfu_gb300.so`` (in-tree, git-ignored),
then the headless C++ frame loop ``driver/kinfu_run.cpp`` into ``lib/kinfu_run``.

Device code is compiled with ``-fmad=false`` and host code with
``-ffp-contract=off``: the plain FP32 form reproduces the reference's per-element
float arithmetic operation for operation, which only holds when no multiply-add is
fused behind the source's back.  Division and square root stay IEEE round-to-nearest
(nvcc's defaults; no fast-math).
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
INCLUDE = PKG.parent / "include"
OUT_DIR = PKG / "lib"
BUILD_DIR = PKG / "_build"
LIB = OUT_DIR / "libkinfu_gb300.so"
DRIVER_SRC = PKG / "driver" / "kinfu_run.cpp"
DRIVER = OUT_DIR / "kinfu_run"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3", "-std=c++17", "-lineinfo", "-fmad=false", "--prec-div=true", "--prec-sqrt=true",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math", "-I", str(INCLUDE), *ARCH,
]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the kinfu_gb300 library needs the CUDA toolkit to build")
    return cand


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def headers() -> list[Path]:
    return sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + sorted(INCLUDE.glob("*.h"))


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def build_driver(force: bool = False, verbose: bool = False) -> Path:
    """The headless C++ frame loop (driver/kinfu_run.cpp over include/kinfu_pipeline.hpp),
    linked against the library with an $ORIGIN run path."""
    deps = [DRIVER_SRC, LIB, INCLUDE / "kinfu_pipeline.hpp", INCLUDE / "kinfu_gb300.h"]
    if not force and not _stale(DRIVER, deps):
        return DRIVER
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        raise RuntimeError("no C++ compiler for the kinfu_run driver")
    tmp = DRIVER.with_suffix(".tmp")
    cmd = [cxx, "-std=c++17", "-O2", "-Wall", "-I", str(INCLUDE), str(DRIVER_SRC), "-L", str(OUT_DIR),
           "-lkinfu_gb300", "-Wl,-rpath,$ORIGIN", "-o", str(tmp)]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"kinfu_run failed to build:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, DRIVER)
    return DRIVER


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> Path:
    lib = build_library(force, verbose, extra)
    build_driver(force, verbose)
    return lib


def build_library(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> Path:
    srcs = sources()
    deps = srcs + headers() + [Path(__file__)]
    if not force and not _stale(LIB, deps):
        return LIB
    BUILD_DIR.mkdir(exist_ok=True)
    OUT_DIR.mkdir(exist_ok=True)
    cc = nvcc()
    extra = list(extra or [])

    def compile_one(src: Path) -> Path:
        obj = BUILD_DIR / (src.stem + ".o")
        cmd = [cc, *NVCC_FLAGS, *extra, "-c", str(src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr, flush=True)
        return obj

    with ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [cc, "-shared", *ARCH, "-o", str(tmp), *map(str, objs), "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv,
                extra=["-Xptxas", "-v"] if "--ptxas" in sys.argv else None))
