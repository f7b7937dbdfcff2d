"""Builds the native library libpvglu.so in-tree (sm_103a only).

Compiles the host C++ (symbolic analysis, plant generator) with g++ and the
CUDA translation unit with nvcc for ``-gencode arch=compute_103a,code=sm_103a``
in parallel, then links one shared library next to this file.  No CMake.
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
ROOT = PKG.parent
BUILD = ROOT / "_build"
LIB = PKG / "libpvglu.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code contracts no a*b+c into FMA, so x86-64 and aarch64 builds round alike.
CXXFLAGS = ["-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall", "-Wextra",
            "-Wno-unused-parameter"]
NVCCFLAGS = ["-std=c++17", "-O3", "-lineinfo", "--expt-relaxed-constexpr",
             "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
             "-Xptxas", "-warn-spills"] + ARCH

HOST_SOURCES = ["symbolic.cpp", "symbolic_io.cpp", "programs.cpp", "plant.cpp", "plant_capi.cpp"]
CUDA_SOURCES = ["capi.cu", "newton.cu"]
# newton.cu evaluates the panel model (panel_model.h) on the device; without
# multiply-add contraction it rounds exactly like the host code.
EXTRA_NVCCFLAGS = {"newton.cu": ["--fmad=false"]}


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build pvglu")


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    nvcc = _nvcc()
    headers = list(CSRC.glob("*.h*")) + list(CSRC.glob("*.cuh")) + list((ROOT / "include").glob("*.h"))
    jobs = []
    objs = []
    for src in HOST_SOURCES:
        obj = BUILD / (src + ".o")
        objs.append(obj)
        if force or _stale(obj, [CSRC / src] + headers):
            jobs.append(["g++", *CXXFLAGS, "-I", str(CSRC), "-c", str(CSRC / src), "-o", str(obj)])
    for src in CUDA_SOURCES:
        obj = BUILD / (src + ".o")
        objs.append(obj)
        if force or _stale(obj, [CSRC / src] + headers):
            jobs.append([nvcc, *NVCCFLAGS, *EXTRA_NVCCFLAGS.get(src, []), "-I", str(CSRC), "-c",
                         str(CSRC / src), "-o", str(obj)])
    with ThreadPoolExecutor(max_workers=max(2, len(jobs))) as ex:
        for cmd, _ in zip(jobs, ex.map(_run, jobs)):
            if verbose:
                print(" ".join(cmd), file=sys.stderr)
    if force or jobs or _stale(LIB, objs):
        _run([nvcc, "-shared", *ARCH, "-o", str(LIB), *map(str, objs), "-lcudart"])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
