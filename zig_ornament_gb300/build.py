"""Builds libornament_cuda.so in-tree for sm_103a.

Kernel translation units are compiled by nvcc with
``-gencode arch=compute_103a,code=sm_103a -fmad=false`` (no multiply-add
contraction: the kernels keep the reference's rounding sequence), the host
BVH builder by g++, all in parallel, then linked into
``zig_ornament_gb300/libornament_cuda.so`` with the static CUDA runtime.
A build is skipped when the library is newer than every source and header.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
BUILD = PKG / "_build"
LIB = PKG / "libornament_cuda.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off", f"-I{INCLUDE}", f"-I{CSRC}"]
CXX_FLAGS = ["-std=c++17", "-O2", "-fPIC", "-pthread", "-ffp-contract=off", f"-I{INCLUDE}", f"-I{CSRC}"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libornament_cuda")


def _sources():
    cu = sorted(CSRC.glob("*.cu"))
    cpp = sorted(CSRC.glob("*.cpp"))
    return cu, cpp


def _newest_input() -> float:
    files = list(CSRC.glob("*")) + list(INCLUDE.glob("*.h")) + [Path(__file__)]
    return max(f.stat().st_mtime for f in files if f.is_file())


def _run(cmd):
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(map(str, cmd)) + "\n" + res.stdout + res.stderr)
    return res.stdout + res.stderr


def build_library(force: bool = False, verbose: bool = False) -> Path:
    """Compiles and links libornament_cuda.so; returns its path."""
    if not force and LIB.exists() and LIB.stat().st_mtime >= _newest_input():
        build_driver()
        return LIB
    BUILD.mkdir(exist_ok=True)
    nvcc = _nvcc()
    cu, cpp = _sources()
    jobs = []
    for src in cu:
        obj = BUILD / (src.name + ".o")
        extra = ["-Xptxas", "-v"] if verbose else []
        jobs.append([nvcc, *NVCC_FLAGS, *ARCH, *extra, "-c", str(src), "-o", str(obj)])
    for src in cpp:
        obj = BUILD / (src.name + ".o")
        jobs.append(["g++", *CXX_FLAGS, "-c", str(src), "-o", str(obj)])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            sys.stdout.write(o)
    objs = [str(BUILD / (s.name + ".o")) for s in cu + cpp]
    tmp = LIB.with_suffix(".so.tmp")
    _run([nvcc, "-shared", *ARCH, "-o", str(tmp), *objs, "-lpthread", "-ldl", "-lrt"])
    os.replace(tmp, LIB)
    build_driver(force=True)
    return LIB


DRIVER_SRC = PKG / "driver" / "orn_headless.c"
DRIVER = PKG / "orn_headless"


def build_driver(force: bool = False) -> Path:
    """The plain-C headless frame loop (driver/orn_headless.c), linked
    against the in-tree library with an $ORIGIN rpath."""
    if not force and DRIVER.exists() and DRIVER.stat().st_mtime >= max(
            DRIVER_SRC.stat().st_mtime, LIB.stat().st_mtime):
        return DRIVER
    _run(["gcc", "-std=c11", "-O2", "-Wall", "-Wextra", "-D_POSIX_C_SOURCE=200809L", f"-I{INCLUDE}",
          str(DRIVER_SRC), "-o", str(DRIVER), f"-L{PKG}", "-lornament_cuda", "-Wl,-rpath,$ORIGIN", "-lm"])
    return DRIVER


if __name__ == "__main__":
    p = build_library(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(p)
