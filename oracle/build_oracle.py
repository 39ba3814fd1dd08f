"""Build recipe for the CPU oracles (test infrastructure).

liboracle.so (the restatement, oracle/oracle.cpp) is always built into
oracle/_build/.  When the zig_ornament sources are present (the directory in
ORN_REFERENCE_DIR, default /root/reference), the reference's own HIP kernel
source is compiled unmodified through oracle/shim into
oracle/_ref/libref_libm.so (glibc transcendentals) and
oracle/_ref/libref_pmath.so (the project's portable transcendentals).
All three use the same flags: -O3 -ffp-contract=off -fno-fast-math (no
multiply-add contraction, as on the GPU) with OpenMP, so the restatement and
the reference's code are timed on equal terms.  No -march/-mcpu=native: the
same objects must give the same bits on x86-64 and aarch64 hosts.

This recipe is the one place that names where the reference sources are
looked for: ORN_REFERENCE_DIR when set, else the checkout location of the
build container.
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
BUILD = HERE / "_build"
REF_OUT = HERE / "_ref"
ORACLE_LIB = BUILD / "liboracle.so"
REF_LIBM = REF_OUT / "libref_libm.so"
REF_PMATH = REF_OUT / "libref_pmath.so"
REFERENCE_DIR = Path(os.environ.get("ORN_REFERENCE_DIR", "/root/reference"))
REF_KERNELS = REFERENCE_DIR / "src" / "hip_backend" / "kernels"

FLAGS = ["-std=c++17", "-O3", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared",
         f"-I{ROOT / 'include'}", f"-I{ROOT / 'zig_ornament_gb300' / 'csrc'}"]


def _newer(out: Path, inputs) -> bool:
    return out.exists() and all(out.stat().st_mtime >= Path(i).stat().st_mtime for i in inputs)


def _cc(args):
    r = subprocess.run(["g++", *args], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + " ".join(args) + "\n" + r.stderr)


def build_oracle(force: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    src = HERE / "oracle.cpp"
    deps = [src, ROOT / "zig_ornament_gb300" / "csrc" / "pmath.h", ROOT / "include" / "ornament_cuda.h",
            Path(__file__)]
    if force or not _newer(ORACLE_LIB, deps):
        _cc([*FLAGS, str(src), "-o", str(ORACLE_LIB)])
    return ORACLE_LIB


def reference_available() -> bool:
    return (REF_KERNELS / "pathtracer.hip.cpp").exists()


def build_ref(force: bool = False):
    """Compiles the reference kernels for the host; returns the two library
    paths, or None when the reference sources are not present."""
    if not reference_available():
        return None
    REF_OUT.mkdir(exist_ok=True)
    src = HERE / "ref_driver.cpp"
    deps = [src, *sorted((HERE / "shim").rglob("*.h")), ROOT / "zig_ornament_gb300" / "csrc" / "pmath.h",
            Path(__file__)]
    inc = ["-I" + str(HERE / "shim"), "-I" + str(REF_KERNELS)]
    for out, extra in ((REF_LIBM, []), (REF_PMATH, ["-DORN_SHIM_PORTABLE_MATH"])):
        if force or not _newer(out, deps):
            _cc([*FLAGS, *inc, *extra, str(src), "-o", str(out)])
    return REF_LIBM, REF_PMATH


if __name__ == "__main__":
    print(build_oracle(force=True))
    print(build_ref(force=True))
