"""Speed of the CPU restatement (oracle/oracle.cpp) against the reference's
own kernels compiled for the host (oracle/_ref), on the same cores, pixels
and flags (oracle/build_oracle.py: -O3 -ffp-contract=off, OpenMP).

Test infrastructure, run where the reference sources are present:

    python oracle/port_speed.py [--width 480 --height 270 --spp 2]

It renders the 1080p instanced-mesh workload's scene (at a smaller
resolution, same geometry, camera and depth 8) with
  * the reference's kernels with glibc transcendentals (libref_libm.so: the
    reference as a host compiler builds it),
  * the reference's kernels with the project's portable transcendentals
    (libref_pmath.so), and
  * the restatement with the portable transcendentals (liboracle.so: what
    bench.py times as the CPU baseline and the reference arm),
all threads and one thread, checks that the restatement's accumulation is
bit-identical to libref_pmath's, and writes the rates and the ratio
restatement / reference to oracle/port_speed.json, which bench.py quotes in
its cpu_baseline (the GPU host cannot build the reference: its sources are
not there).
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))

OUT = HERE / "port_speed.json"


def _cpu_name() -> str:
    try:
        for line in Path("/proc/cpuinfo").read_text().splitlines():
            if line.lower().startswith(("model name", "cpu model")):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.processor() or platform.machine()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--width", type=int, default=480)
    ap.add_argument("--height", type=int, default=270)
    ap.add_argument("--spp", type=int, default=2)
    ap.add_argument("--repeats", type=int, default=3)
    args = ap.parse_args()

    from oracle import build_oracle as bo
    from oracle import oracle_lib as ol
    from zig_ornament_gb300 import ornament, scenes

    if not ol.reference_available():
        raise SystemExit("zig_ornament sources not found: set ORN_REFERENCE_DIR")
    W, H, spp = args.width, args.height, args.spp
    scene = scenes.instanced_meshes_scene(W, H)
    bvh = ornament.Bvh(scene, row_major_transforms=True)
    cp = ol.make_params(scene.camera, W, H, depth=8, textures_count=bvh.scene_textures_count)
    oracle = ol.Oracle()
    ref_libm = ol.Reference(portable_math=False)
    ref_pmath = ol.Reference(portable_math=True)
    cores = os.cpu_count() or 1

    def rate(fn, threads):
        best = []
        for _ in range(args.repeats):
            t0 = time.perf_counter()
            fn(threads)
            best.append(time.perf_counter() - t0)
        return W * H * spp / float(np.median(best)) / 1e6

    runs = {
        "reference_glibc_math": lambda t: ref_libm.render(bvh, cp, spp, threads=t),
        "reference_portable_math": lambda t: ref_pmath.render(bvh, cp, spp, threads=t),
        "restatement": lambda t: oracle.render(bvh, cp, spp, portable_math=True, threads=t),
    }
    # same bits: the restatement against the reference with the same transcendentals
    a_ref, _, _ = ref_pmath.render(bvh, cp, spp, threads=cores)
    a_port, _, _, _ = oracle.render(bvh, cp, spp, portable_math=True, threads=cores)
    identical = bool(np.array_equal(a_ref.view(np.uint32), a_port.view(np.uint32)))
    res = {"all_threads": {}, "one_thread": {}}
    for name, fn in runs.items():
        res["all_threads"][name] = round(rate(fn, cores), 4)
        res["one_thread"][name] = round(rate(fn, 1), 4)
    out = {
        "what": "Msamples/s of the CPU restatement and of the reference's own kernels compiled for the host",
        "host": {"machine": platform.machine(), "cpu": _cpu_name(), "cores": cores},
        "flags": " ".join(f for f in bo.FLAGS if f.startswith(("-O", "-ff", "-fno", "-fopenmp"))),
        "workload": f"instanced-mesh scene, {W}x{H}, {spp} spp, depth 8, median of {args.repeats}",
        "msamples_per_s": res,
        "accumulation_bit_identical": identical,
        "restatement_over_reference": {
            k: round(res[k]["restatement"] / res[k]["reference_glibc_math"], 3) for k in res},
        "restatement_over_reference_same_math": {
            k: round(res[k]["restatement"] / res[k]["reference_portable_math"], 3) for k in res},
    }
    OUT.write_text(json.dumps(out, indent=1) + "\n")
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    main()
