"""Benchmark: Msamples/s of the plain megakernel on the 1080p instanced-mesh
scene (8 BLAS of 10k-80k triangles, 256 instances, 4 textures, one emissive
quad, 1920x1080, 256 spp, depth 8), on 1..N GB300s.

One step = one PathTracer.render() of `--spp` sample passes (default 256,
the configuration's sample count) continuing the progressive render.

  value    Msamples/s with the scene and targets resident in HBM; device time
           of each step from CUDA events on the library's stream; L2 is
           flushed (a 256 MiB write) between timed steps, outside the events.
  e2e      the same metric through the C ABI as an application uses it:
           orn_render + orn_get_framebuffer into pinned host memory each step
           (the 144-byte ConstantParams go host-to-device with the launch; the
           1080p RGBA32F framebuffer comes back), timed by CUDA events.
  roofline algorithmic bytes per megakernel launch from exact work counters
           of one extra (untimed) step — node visits, leaf transforms, hit
           shading gathers, per-sample buffer traffic — over the average
           launch time.  The L2-resident scenes are bound by the L1/TEX
           pipeline and issue slots: `bound` "l1tex", against the nominal L1
           load bandwidth, with the ncu figures of this build (SOL
           percentages, active threads per warp) and the HBM share beside
           it; the large scene is bound by HBM latency: `bound` "hbm",
           DRAM traffic against the measured copy bandwidth.  ncu figures
           come from the committed profiles/ summary of the same kernel
           sources (null when the sources changed since that capture).
  cpu_baseline  the CPU restatement of the reference (oracle/oracle.cpp, all
           host threads, -O3) on a bounded sample of the same workload, with
           its measured speed relative to the reference's own kernels
           (oracle/port_speed.json).

`--impl reference` times the reference implementation of the path on the
host cores (the CPU restatement, pinned bit-for-bit to the reference's own
kernels) on the same workload sample; it runs on rank 0 only.

Multi-GPU: one process per GPU (torchrun); every rank renders its own copy
of the frame (replicas: pixels and samples are independent, no exchange);
value = all ranks' samples / the slowest rank's time.

The headline line also carries: the same steps on the non-parity trees
(`sah_tree`, `lbvh_tree`); the same steps on the persistent wavefront with
its autotuned launch parameters (`wavefront`, same images);
`configs` — the sphere field (640x360, 64 spp),
the large scene (3840x2160, 16 spp, depth 16) and the 64-scene batch (every
scene's full sample count, one graph-replayed launch against one launch per
scene), each with rays/s, roofline and CPU baseline; and `time_to_relmse` —
plain tracing on the parity and SAH trees against the cached renderers, to
relMSE 1e-3 against a 16k-sample FP64 oracle, on the radiance-cache
configuration at 1920x1080 and a closed room at 640x360.  Other modes:
`--workload spheres|large`, `--bvh sah|lbvh`, `--kernel wavefront` (after
orn_wave_tune unless `--no-wave-tune`),
`--mode relmse` (the block alone; `--workload large` for the large scene at
960x540), `--mode batch`, `--mode cached-frames [--batched]` (a profiling
workload of radiance-cache frames).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Msamples/s at 1080p"
UNIT = "Msamples/s"
TREE_SUFFIX = {"reference": "", "sah": ", SAH tree", "lbvh": ", LBVH tree"}
TREE_DESC = {"reference": "bvh.zig rules (random axis, median split): the parity tree",
             "sah": "binned SAH (non-parity mode)",
             "lbvh": "GPU-built linear BVH BLASes + SAH TLAS (non-parity mode)"}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--workload", default="instanced", choices=["instanced", "spheres", "large"],
                   help="instanced: the 1080p instanced-mesh scene (default, the headline); spheres: the "
                        "640x360 sphere field (64 spp, depth 10); large: 4096 instances over ~10M "
                        "triangles at 3840x2160 (depth 16)")
    p.add_argument("--bvh", default="reference", choices=["reference", "sah", "lbvh"],
                   help="reference: bvh.zig's tree (the parity tree, default); sah: the binned-SAH tree; "
                        "lbvh: BLASes built on the GPU as linear BVHs, TLAS by SAH (both non-parity modes: "
                        "fewer node visits, images equal in expectation)")
    p.add_argument("--spp", type=int, default=None, help="sample passes per step (render iterations)")
    p.add_argument("--width", type=int, default=None)
    p.add_argument("--height", type=int, default=None)
    p.add_argument("--depth", type=int, default=None)
    p.add_argument("--cpu-seconds", type=float, default=15.0, help="target length of the CPU baseline sample")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--kernel", default="mega", choices=["mega", "wavefront"])
    p.add_argument("--mode", default="throughput", choices=["throughput", "relmse", "cached-frames", "batch"],
                   help="throughput: the Msamples/s line (with the time-to-relMSE block unless "
                        "--no-relmse); relmse: only the time-to-relMSE measurement; cached-frames: "
                        "render --frames radiance-cache frames (a profiling workload); batch: the 64-scene "
                        "batched renderer against one launch per scene")
    p.add_argument("--batch-scenes", type=int, default=64)
    p.add_argument("--batch-spp-divisor", type=int, default=16,
                   help="batch: each frame renders spp/divisor of every scene's 16-256 samples")
    p.add_argument("--tune-cache", default=None, help="batch: autotuner JSON cache (default: none)")
    p.add_argument("--no-relmse", action="store_true", help="skip the time-to-relMSE block")
    p.add_argument("--no-sah-line", action="store_true", help="skip the SAH-tree figure")
    p.add_argument("--no-wavefront-line", action="store_true",
                   help="skip the persistent wavefront's figure in the headline line")
    p.add_argument("--no-wave-tune", action="store_true",
                   help="--kernel wavefront: keep the default launch parameters instead of orn_wave_tune's")
    p.add_argument("--no-configs", action="store_true",
                   help="skip the other configurations (sphere field, 64-scene batch, large scene)")
    p.add_argument("--relmse-width", type=int, default=1920)
    p.add_argument("--relmse-height", type=int, default=1080)
    p.add_argument("--relmse-target", type=float, default=1e-3)
    p.add_argument("--relmse-ref-spp", type=int, default=16384)
    p.add_argument("--relmse-budget", type=float, default=12.0, help="GPU seconds per method at most")
    p.add_argument("--frames", type=int, default=8, help="cached-frames: timed frames")
    p.add_argument("--batched", action="store_true",
                   help="cached-frames: the cached + batched configuration of the relMSE harness (8 sample "
                        "streams, Sobol sampler, SAH tree, train_shift 3, lr 5e-3, 64 steps per frame)")
    p.add_argument("--scene", default="instanced", choices=["instanced", "closed-room"],
                   help="cached-frames: the scene")
    p.add_argument("--cached-kernel", default="mega", choices=["mega", "wavefront"],
                   help="the cached renderer's kernel (relmse and cached-frames): the megakernel "
                        "(KERNEL_CACHED, the faster) or the persistent wavefront (KERNEL_CACHED_WAVEFRONT)")
    return p.parse_args()


# Per-workload defaults: (width, height, spp per step, depth).
WORKLOAD_DEFAULTS = {"instanced": (1920, 1080, 256, 8), "spheres": (640, 360, 64, 10), "large": (3840, 2160, 16, 16)}


def apply_workload_defaults(args):
    w, h, spp, depth = WORKLOAD_DEFAULTS[args.workload]
    args.width = args.width or w
    args.height = args.height or h
    args.spp = args.spp or spp
    args.depth = args.depth or depth
    return args


def metric_name(args):
    if args.workload == "instanced" and (args.width, args.height) == (1920, 1080) and args.bvh == "reference":
        return METRIC
    return f"Msamples/s, {args.workload} {args.width}x{args.height}" + TREE_SUFFIX[args.bvh]


def workload(args):
    from zig_ornament_gb300 import scenes, ornament
    if args.workload == "spheres":
        scene = scenes.spheres_scene(args.width, args.height)
        desc = ("sphere field: ground r=1000, 3 r=1 spheres, 22x22 grid of r=0.2 spheres (80% lambertian, "
                "15% metal, 5% dielectric), sky gradient, aperture 0.1")
    elif args.workload == "large":
        scene = scenes.large_scene(args.width, args.height)
        desc = ("large: 4096 instances over 32 BLAS icospheres+tori (~10M tris), 40% dielectric / 30% metal "
                "(fuzz U(0,0.3)) / 30% textured lambertian, 4 procedural 1024^2 textures, 8 emissive quads, "
                "instances in a 250^3 box (the 1080p scene's density)")
    else:
        scene = scenes.instanced_meshes_scene(args.width, args.height)
        desc = ("instanced meshes TLAS/BLAS: 8 BLAS icospheres+tori 10k-80k tris, 256 instances, "
                "4 procedural 1024^2 RGBA8 textures, 1 emissive quad (radiance 15)")
    t_build = time.perf_counter()
    bvh = ornament.Bvh(scene, builder=args.bvh)
    t_build = time.perf_counter() - t_build
    tris = sum(len(m.vertex_indices) // 3 for m in scene.meshes)
    cfg = {"workload": desc, "bvh": TREE_DESC[args.bvh], "bvh_build_s": round(t_build, 3),
           "resolution": f"{args.width}x{args.height}", "spp_per_step": args.spp, "depth": args.depth,
           "triangles": tris, "instances": len(scene.mesh_instances), "blas": len(scene.meshes),
           "tlas_nodes": int(len(bvh.tlas_nodes)), "blas_nodes": int(len(bvh.blas_nodes)),
           "kernel": ("plain megakernel (persistent, warp-synchronous, passes looped per pixel)"
                      if args.kernel == "mega" else "persistent wavefront (per-block path pools, ray and hit "
                                                   "queues in shared memory, warps traverse or shade)"),
           "semantics": "HIP", "transcendentals": "portable (bit-exact with the CPU oracle)",
           "l2": "flushed between timed steps (256 MiB write)", "parallelism": "replicas"}
    return scene, bvh, cfg


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def algorithmic_bytes(c):
    """Bytes the algorithm touches, from exact work counters (per the
    reference's data layout): 64 B per node visit, 64 B inverse transform per
    sphere-leaf test and per mesh entry, 32 B material per hit, 64 B forward
    transform per sphere hit, 96 B index/normal/uv gathers plus a 64 B
    inverse transform per mesh hit, 4 B per textured hit, and per sample
    16 B accumulation read + 16 B write + 8 B RNG read/write + 16 B
    framebuffer."""
    hits = c["sphere_hits"] + c["mesh_hits"]
    return (64 * c["visits"] + 64 * (c["sphere_leaf"] + c["mesh_entry"]) + 32 * hits + 64 * c["sphere_hits"]
            + (96 + 64) * c["mesh_hits"] + 4 * c["textured_hits"] + 56 * c["samples"])


def cpu_baseline(bvh, scene, args, seconds, threads=0):
    """The CPU restatement on the host cores over every k-th pixel of the
    frame, k chosen for about `seconds` of work; returns (Msamples/s,
    threads, description)."""
    from oracle import oracle_lib as ol
    oracle = ol.Oracle()
    cp = ol.make_params(scene.camera, args.width, args.height, depth=args.depth,
                        textures_count=bvh.scene_textures_count)
    n = args.width * args.height
    nthreads = threads or os.cpu_count() or 1
    spp = 4
    # calibrate on every 256th pixel, then size the stride for the budget
    t0 = time.perf_counter()
    oracle.render(bvh, cp, 1, pixel_range=(0, n), pixel_stride=256, threads=nthreads)
    rate = (n // 256) / max(time.perf_counter() - t0, 1e-6)
    stride = max(1, int(n * spp / max(rate * seconds, 1.0)))
    if stride == 1:   # a cheap frame: more passes over every pixel instead
        spp = max(spp, int(rate * seconds / n))
    pixels = (n + stride - 1) // stride
    t0 = time.perf_counter()
    oracle.render(bvh, cp, spp, pixel_range=(0, n), pixel_stride=stride, threads=nthreads)
    dt = time.perf_counter() - t0
    value = pixels * spp / dt / 1e6
    return value, nthreads, f"every {stride}th pixel of the frame ({pixels} pixels) x {spp} spp, {dt:.1f} s"


def source_hash(files=None):
    """Hash of kernel sources and the build flags: `files` (paths relative to
    the repository: the translation units and headers of one kernel and its
    host launcher), or every file of csrc/ and include/ plus build.py.
    Identifies the build an ncu capture was taken of."""
    import hashlib
    h = hashlib.sha256()
    if files is None:
        paths = (sorted((ROOT / "zig_ornament_gb300" / "csrc").glob("*")) + sorted((ROOT / "include").glob("*.h"))
                 + [ROOT / "zig_ornament_gb300" / "build.py"])
    else:
        paths = [ROOT / f for f in files]
    for f in paths:
        if f.is_file():
            h.update(f.name.encode())
            h.update(f.read_bytes())
        else:
            h.update(b"missing:" + str(f.name).encode())
    return h.hexdigest()[:16]


def profile_figures(name):
    """(figures, source) of a committed ncu summary, profiles/<name>.md, whose
    `figures:` line holds the counters bench.py quotes (DRAM bytes per node
    visit, SOL percentages) and the source files the captured kernel was
    built from; figures is None unless those files are unchanged since the
    capture (source_hash)."""
    p = ROOT / "profiles" / f"{name}.md"
    if not p.exists():
        return None, f"profiles/{name}.md absent"
    for line in p.read_text().splitlines():
        if line.strip().startswith("figures:"):
            try:
                d = json.loads(line.split(":", 1)[1])
            except ValueError:
                return None, f"profiles/{name}.md: unreadable figures line"
            if d.get("sources") != source_hash(d.get("files")):
                return None, f"profiles/{name}.md was captured from other kernel sources"
            return d, f"profiles/{name}.md (ncu, this build)"
    return None, f"profiles/{name}.md has no figures line"


# The sources of the megakernel and its launcher (profile figures lines).
MEGA_SOURCES = ["zig_ornament_gb300/csrc/" + f for f in (
    "megakernel.cu", "pt_device.cuh", "pt_machine.cuh", "pt_kernels.h", "pt_scene.h", "pmath.h", "qmc.cuh",
    "capi.cu", "order.cu")] + ["include/ornament_cuda.h", "zig_ornament_gb300/build.py"]


def l1_peak_gbs(clocks, device=0):
    """Nominal L1 load bandwidth of the GPU: 128 bytes per clock per SM at
    the maximum SM clock (not a measured figure)."""
    import torch
    sms = torch.cuda.get_device_properties(device).multi_processor_count
    mhz = (clocks or {}).get("sm_max_mhz") or 2070.0
    return sms * 128 * mhz * 1e6 / 1e9


def roofline_block(bytes_per_launch, avg_launch_s, workload, clocks, profile_name, device=0, visits_per_launch=None):
    """The roofline object of a megakernel workload.

    L2-resident scenes (every workload but `large`): the kernel is bound by
    the L1/TEX pipeline and issue slots (ncu: L1/TEX throughput and issue
    activity near 60 %, DRAM below 1 %), so `achieved` (algorithmic bytes per
    launch over the measured launch time) is set against the nominal L1 load
    bandwidth, and the ncu figures of this build are quoted beside it.
    The large scene (1.3 GB of nodes, L2 hit rate ~60 %) is bound by HBM
    latency: `achieved` is the DRAM traffic of one launch over the launch
    time, against the measured HBM copy bandwidth.  `traffic` = DRAM bytes
    per node visit of the ncu capture of this build (a smaller launch of the
    same scene) x this launch's node visits."""
    peak_hbm, kind = measured_peaks()
    algo = bytes_per_launch / avg_launch_s / 1e9
    fig, src = profile_figures(profile_name) if profile_name else (None, "no profile")
    traffic = None
    if fig and "dram_bytes_per_visit" in fig and visits_per_launch:
        traffic = fig["dram_bytes_per_visit"] * visits_per_launch
    hbm = {"achieved": traffic / avg_launch_s / 1e9 if traffic else None, "peak": peak_hbm, "unit": "GB/s",
           "peak_kind": f"{kind} HBM copy"}
    hbm["frac"] = hbm["achieved"] / peak_hbm if hbm["achieved"] else None
    if workload == "large":
        out = {"bound": "hbm", "achieved": hbm["achieved"], "peak": peak_hbm, "unit": "GB/s", "frac": hbm["frac"],
               "traffic": traffic, "peak_kind": f"{kind} HBM copy",
               "algorithmic": {"achieved": algo, "unit": "GB/s",
                               "note": "node and shading bytes the algorithm reads, L1/L2-served ones included"}}
    else:
        l1 = l1_peak_gbs(clocks, device)
        out = {"bound": "l1tex", "achieved": algo, "peak": l1, "unit": "GB/s", "frac": algo / l1,
               "traffic": traffic, "peak_kind": "nominal L1 load bandwidth (128 B/clk/SM x SMs x max SM clock)",
               "hbm": hbm}
    out["ncu"] = ({k: fig[k] for k in fig if k not in ("sources",)} if fig else None)
    out["ncu_source"] = src
    return out


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    scene, bvh, cfg = workload(args)
    vals = []
    desc = ""
    for i in range(args.warmup + args.steps):
        v, cores, desc = cpu_baseline(bvh, scene, args, max(2.0, args.cpu_seconds / 3))
        if i >= args.warmup:
            vals.append(v)
    value = float(np.median(vals))
    line = {"impl": "reference", "metric": metric_name(args), "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)", "config": cfg,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": "per step: " + desc + "; the CPU restatement of the reference's HIP "
                                       "kernels (bit-exact with them), OpenMP over pixels"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def reduce_max(values, dist, device="cpu"):
    """Max over ranks of each timing (the slowest rank bounds the job)."""
    if dist is None:
        return [float(v) for v in values]
    import torch
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t.tolist()]


def job_throughput(world, samples_per_step, steps, total_ms):
    """Whole-job Msamples/s: every rank renders its own replica of the frame."""
    return world * samples_per_step * steps / (total_ms / 1e3) / 1e6


def run_ours(args):
    import torch
    from zig_ornament_gb300 import _lib, ornament

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    scene, bvh, cfg = workload(args)
    r = ornament.Renderer(bvh, device=local)
    r.set_resolution(args.width, args.height)
    st = _lib.State()
    st.depth, st.flip_y, st.inverted_gamma, st.iterations = args.depth, 0, 1.0, args.spp
    st.ray_cast_epsilon, st.semantics, st.spp_per_launch = 0.001, 0, 0
    st.kernel = _lib.KERNEL_WAVEFRONT if args.kernel == "wavefront" else _lib.KERNEL_MEGA
    r.set_state(st)
    r.set_camera(scene.camera.to_struct())
    if args.kernel == "wavefront":
        # the autotuner picks the block shape, fetch threshold and round
        # length for this scene and resolution (untimed; scratch targets)
        t_tune = time.perf_counter()
        wave_cfg = r.wave_config() if args.no_wave_tune else r.wave_tune()
        cfg["wave_config"] = {**wave_cfg, "tune_s": round(time.perf_counter() - t_tune, 2)}
    stream = torch.cuda.ExternalStream(r.stream(), device=torch.device("cuda", local))
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    n_px = args.width * args.height
    fb_host = torch.empty((n_px, 4), dtype=torch.float32, pin_memory=True)
    fb_np = fb_host.numpy()

    def barrier():
        torch.cuda.synchronize()
        if dist:
            dist.barrier()

    def flush_l2():
        with torch.cuda.stream(stream):
            flush.zero_()

    for _ in range(args.warmup):
        r.render()
        flush_l2()
    r.synchronize()
    launches0 = r.launch_count()
    barrier()
    times = []
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            r.render()
            e1.record(stream)
            flush_l2()
            times.append((e0, e1))
        r.synchronize()
        torch.cuda.synchronize()
    barrier()
    step_ms = [a.elapsed_time(b) for a, b in times]
    launches = r.launch_count() - launches0
    # e2e: render + framebuffer readback through the C ABI, host buffers
    e2e_times = []
    for _ in range(args.steps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        r.render()
        r.framebuffer(fb_np)
        e1.record(stream)
        flush_l2()
        e2e_times.append((e0, e1))
    r.synchronize()
    e2e_ms = [a.elapsed_time(b) for a, b in e2e_times]
    # exact work of one step (untimed)
    r.enable_counters(True)
    r.render()
    counters = r.counters()
    r.enable_counters(False)
    launches_per_step = launches / args.steps
    samples_step = n_px * args.spp
    total_ms = float(sum(step_ms))
    total_e2e = float(sum(e2e_ms))
    total_ms, total_e2e = reduce_max([total_ms, total_e2e], dist, device=f"cuda:{local}")
    value = job_throughput(world, samples_step, args.steps, total_ms)
    e2e_value = job_throughput(world, samples_step, args.steps, total_e2e)
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return
    avg_launch_s = (sum(step_ms) / 1e3) / max(launches, 1)
    bytes_per_launch = algorithmic_bytes(counters) / max(launches_per_step, 1)
    clk = clocks.summary()
    line = {
        "metric": metric_name(args), "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)",
        "config": cfg,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 144 * launches_per_step,
                "d2h_bytes_per_step": n_px * 16},
        "gpu_launches": int(launches),
        "rays_per_s": counters["rays"] / samples_step * value * 1e6,
        "work_per_step": counters,
        "roofline": roofline_block(bytes_per_launch, avg_launch_s, args.workload, clk,
                                   PROFILE_OF_WORKLOAD.get(args.workload if args.kernel == "mega" else "wavefront"),
                                   local, counters["visits"] / max(launches_per_step, 1)),
        "clocks": clk,
    }
    headline = args.kernel == "mega" and args.bvh == "reference" and metric_name(args) == METRIC
    if headline and not args.no_sah_line:
        # the same steps on the non-parity trees, for reference
        for alt in ("sah", "lbvh"):
            key = alt + "_tree"
            try:
                t_alt = time.perf_counter()
                alt_bvh = ornament.Bvh(scene, builder=alt)
                t_alt = time.perf_counter() - t_alt
                m = measure_render(alt_bvh, scene, args.width, args.height, args.spp, args.depth,
                                   args.steps, args.warmup, local, flush)
                line[key] = {"value": m["value"], "unit": UNIT, "bvh_build_s": round(t_alt, 3),
                             "note": f"same steps on the {TREE_DESC[alt]} tree: images equal to the "
                                     "reference's in expectation only"}
            except Exception as exc:
                line[key] = {"error": f"{type(exc).__name__}: {exc}"}
    if headline and not args.no_wavefront_line:
        # the same steps on the persistent wavefront (same images), with the
        # launch parameters its autotuner picks for this workload
        try:
            m = measure_render(bvh, scene, args.width, args.height, args.spp, args.depth, args.steps,
                               args.warmup, local, flush, kernel="wavefront")
            line["wavefront"] = {"value": m["value"], "unit": UNIT, "vs_megakernel": m["value"] / value,
                                 "ms_per_step": m["ms_per_step"], "launches_per_step": m["launches_per_step"],
                                 "wave_config": m["wave_config"],
                                 "note": "persistent wavefront (ORN_KERNEL_WAVEFRONT), bit-identical images; "
                                         "device time of the same renders, L2 flushed between them"}
        except Exception as exc:
            line["wavefront"] = {"error": f"{type(exc).__name__}: {exc}"}
    if not args.no_cpu_baseline:
        v, cores, desc = cpu_baseline(bvh, scene, args, args.cpu_seconds)
        v1, _, desc1 = cpu_baseline(bvh, scene, args, 4.0, threads=1)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                                "sample": desc + "; CPU restatement of the reference (bit-exact with its own "
                                          "kernels compiled for the host)",
                                "single_thread": {"value": v1, "sample": desc1}, **port_speed_note()}
    if headline and not args.no_configs:
        line["configs"] = other_configs(args, local, flush)
    if headline and not args.no_relmse:
        try:
            line["time_to_relmse"] = relmse_block(args)
        except Exception as exc:   # the throughput line stands on its own
            line["time_to_relmse"] = {"error": f"{type(exc).__name__}: {exc}"}
    print(json.dumps(line), flush=True)
    r.close()
    if dist:
        dist.destroy_process_group()


# Committed ncu summary (profiles/<name>.md) of each workload's render kernel.
PROFILE_OF_WORKLOAD = {"instanced": "mega_kernel_1080p_32spp", "spheres": "mega_kernel_spheres_640x360",
                       "large": "mega_kernel_large_960x540", "wavefront": "wave_kernel_1080p"}


def port_speed_note():
    """The restatement's flags and its measured speed relative to the
    reference's own kernels (oracle/port_speed.py, run where the reference
    sources are; the GPU host has no copy of them)."""
    from oracle import build_oracle as bo
    note = {"flags": " ".join(f for f in bo.FLAGS if f.startswith(("-O", "-ff", "-fno", "-fopenmp")))}
    p = ROOT / "oracle" / "port_speed.json"
    if p.exists():
        d = json.loads(p.read_text())
        note["port_over_reference"] = {
            "restatement_over_reference": d.get("restatement_over_reference"),
            "restatement_over_reference_same_math": d.get("restatement_over_reference_same_math"),
            "measured_on": d.get("host"), "workload": d.get("workload"), "source": "oracle/port_speed.json"}
    return note


def measure_render(bvh, scene, w, h, spp, depth, steps, warmup, local, flush, counters=False, kernel="mega"):
    """Device time of `steps` renders of `spp` passes (L2 flushed between
    them); returns Msamples/s, ms per step, launches per step and, with
    `counters`, the exact work of one more (untimed) render.  kernel
    "wavefront" renders on the persistent wavefront with the launch
    parameters orn_wave_tune picks (untimed; returned as wave_config)."""
    import torch
    from zig_ornament_gb300 import _lib, ornament
    r = ornament.Renderer(bvh, device=local)
    r.set_resolution(w, h)
    st = _lib.State()
    st.depth, st.flip_y, st.inverted_gamma, st.iterations = depth, 0, 1.0, spp
    st.ray_cast_epsilon, st.semantics, st.spp_per_launch = 0.001, 0, 0
    st.kernel = _lib.KERNEL_WAVEFRONT if kernel == "wavefront" else _lib.KERNEL_MEGA
    r.set_state(st)
    r.set_camera(scene.camera.to_struct())
    wave_cfg = None
    if kernel == "wavefront":
        t_tune = time.perf_counter()
        wave_cfg = {**r.wave_tune(), "tune_s": round(time.perf_counter() - t_tune, 2)}
    stream = torch.cuda.ExternalStream(r.stream(), device=torch.device("cuda", local))

    def flush_l2():
        with torch.cuda.stream(stream):
            flush.zero_()

    for _ in range(warmup):
        r.render()
        flush_l2()
    r.synchronize()
    l0 = r.launch_count()
    ms = []
    for _ in range(steps):
        r.render()
        ms.append(r.last_render_ms())
        flush_l2()
    r.synchronize()
    launches = (r.launch_count() - l0) / steps
    out = {"value": w * h * spp / (float(np.mean(ms)) / 1e3) / 1e6, "ms_per_step": float(np.mean(ms)),
           "launches_per_step": launches}
    if wave_cfg is not None:
        out["wave_config"] = wave_cfg
    if counters:
        r.enable_counters(True)
        r.render()
        out["counters"] = r.counters()
        r.enable_counters(False)
    r.close()
    return out


def other_configs(args, local, flush):
    """The other configurations, compactly: the sphere field (640x360,
    64 spp, depth 10), the 64-scene batch (one persistent launch from a CUDA
    graph against one launch per scene) and the large scene (4096 instances,
    ~10M triangles, 3840x2160, 16 spp, depth 16), each with its rays/s,
    roofline and the CPU restatement on a bounded sample."""
    import copy
    out = {}
    for key, wl, steps, warmup, cpu_s in (("cfg0_spheres", "spheres", 3, 3, 3.0), ("cfg4_large", "large", 2, 1, 4.0)):
        t0 = time.time()
        try:
            a = copy.copy(args)
            a.workload, a.width, a.height, a.spp, a.depth = wl, None, None, None, None
            a = apply_workload_defaults(a)
            scene, bvh, cfg = workload(a)
            m = measure_render(bvh, scene, a.width, a.height, a.spp, a.depth, steps, warmup, local, flush,
                               counters=True)
            c = m["counters"]
            launch_s = m["ms_per_step"] / 1e3 / max(m["launches_per_step"], 1)
            bpl = algorithmic_bytes(c) / max(m["launches_per_step"], 1)
            cpu_v, cores, desc = cpu_baseline(bvh, scene, a, cpu_s)
            out[key] = {"metric": metric_name(a), "value": m["value"], "unit": UNIT,
                        "ms_per_step": m["ms_per_step"], "steps": steps, "warmup": warmup,
                        "rays_per_s": c["rays"] / (a.width * a.height * a.spp) * m["value"] * 1e6,
                        "visits_per_ray": c["visits"] / max(c["rays"], 1),
                        "roofline": roofline_block(bpl, launch_s, wl, None, PROFILE_OF_WORKLOAD[wl], local,
                                                   c["visits"] / max(m["launches_per_step"], 1)),
                        "cpu_baseline": {"value": cpu_v, "unit": UNIT, "cores": cores, "kind": "port",
                                         "sample": desc},
                        "ratio_vs_cpu": m["value"] / cpu_v,
                        "config": {k: cfg[k] for k in ("workload", "resolution", "spp_per_step", "depth",
                                                        "triangles", "instances", "blas_nodes", "bvh_build_s")},
                        "wall_s": round(time.time() - t0, 1)}
        except Exception as exc:
            out[key] = {"error": f"{type(exc).__name__}: {exc}"}
    t0 = time.time()
    try:
        b = copy.copy(args)
        b.steps, b.warmup, b.depth = 1, 1, 8
        out["cfg2_batch"] = batch_measure(b, divisor=1)
        out["cfg2_batch"]["wall_s"] = round(time.time() - t0, 1)
    except Exception as exc:
        out["cfg2_batch"] = {"error": f"{type(exc).__name__}: {exc}"}
    return out


# ---- time to relMSE ------------------------------------------------------------------
def relmse_scene(name, w, h):
    from zig_ornament_gb300 import scenes
    if name == "closed-room":
        return scenes.cornell_box_scene(w, h)
    if name == "large":
        return scenes.large_scene(w, h)
    # the radiance-cache configuration: the 1080p instanced-mesh scene with
    # three emissive quads (rendered at the harness resolution)
    return scenes.instanced_meshes_scene(w, h, n_lights=3)


def crossing_time(curve, target):
    """(seconds, reached) at which a progressive render's relMSE reaches
    `target`, from readings [(seconds, samples, relMSE), ...]: log-linear
    between the two readings around the crossing, the first reading if it is
    already below, or extrapolated as relMSE ~ 1/time when never reached."""
    import math
    reached = curve[-1][2] <= target
    if reached and len(curve) > 1:
        (ta, _, ea), (tb, _, eb) = curve[-2], curve[-1]
        f = (math.log(ea) - math.log(target)) / max(math.log(ea) - math.log(eb), 1e-12)
        return math.exp(math.log(ta) + f * (math.log(tb) - math.log(ta))), True
    if reached:
        return curve[-1][0], True
    return curve[-1][0] * curve[-1][2] / target, False


def time_to_relmse(name, w, h, target, ref_spp, budget_s, depth=8, cache_cfg=None, warmup=64, methods=None,
                   ref=None, streams=8, batched_warmup_spp=16, batched_sobol=True, batched_cfg=None,
                   cached_kernel=None):
    """GPU time each renderer needs to bring the relMSE against an FP64
    `ref_spp`-sample oracle (orn_render_f64 with the plain megakernel on the
    parity tree) down to `target`:
      plain           the plain megakernel on the parity tree (bvh.zig's rules),
      plain_sah       the plain megakernel on the binned-SAH tree, the tree of
                      cached_tuned and cached_batched,
      light_sampling  the cached renderer without the network (every pixel
                      traces its full path with light sampling: unbiased),
      cached          the cached renderer as configured (lr 1e-3, 64 warm-up
                      training frames counted), parity tree,
      cached_tuned    Adam lr 3e-3, 32 warm-up frames, SAH tree,
      cached_batched  `streams` sample streams per pixel batched into each
                      frame's launch (orn_state.spp_per_launch), the Sobol
                      sampler, training slots for 1/8 of the samples at lr
                      5e-3, a 16-sample warm-up, SAH tree;
      cached_batched_wavefront  the same on the persistent wavefront
                      (KERNEL_CACHED_WAVEFRONT; the others use `cached_kernel`,
                      the megakernel by default).
    Progressive rendering in growing chunks; relMSE (orn_relmse, FP64 on the
    GPU) is read between chunks outside the timed renders; the crossing is
    interpolated log-linearly between the two chunks around it, or
    extrapolated as relMSE ~ 1/time past the budget (crossing_time)."""
    from zig_ornament_gb300 import _lib, ornament

    scene = relmse_scene(name, w, h)
    bvh = ornament.Bvh(scene, row_major_transforms=True)
    bvh_sah = None

    def renderer(kernel, tree=None):
        r = ornament.Renderer(tree or bvh, 0)
        r.set_resolution(w, h)
        st = ornament.State()
        st.depth = depth
        st.kernel = kernel
        r.set_state(st.to_struct())
        r.set_camera(scene.camera.to_struct())
        return r, st

    t0 = time.time()
    if ref is None:
        rr, _ = renderer(_lib.KERNEL_MEGA)
        ref = rr.render_f64(ref_spp)
        rr.close()
    ref_s = time.time() - t0
    out = {"resolution": f"{w}x{h}", "depth": depth, "reference_spp": ref_spp, "reference_seconds": round(ref_s, 1),
           "reference": "plain megakernel, parity tree, FP64 accumulation",
           "cached_kernel": "persistent wavefront" if cached_kernel == _lib.KERNEL_CACHED_WAVEFRONT else "megakernel"}
    on_sah = ("plain_sah", "cached_tuned", "cached_batched", "cached_batched_wavefront")
    for method in (methods or ("plain", "plain_sah", "light_sampling", "cached", "cached_tuned", "cached_batched",
                               "cached_batched_wavefront")):
        ck = _lib.KERNEL_CACHED if cached_kernel is None else cached_kernel
        if method == "cached_batched_wavefront":
            ck = _lib.KERNEL_CACHED_WAVEFRONT
        kernel = _lib.KERNEL_MEGA if method in ("plain", "plain_sah") else ck
        batched = method.startswith("cached_batched")
        tuned = method in ("cached_tuned", "cached_batched", "cached_batched_wavefront")
        if method in on_sah and bvh_sah is None:
            bvh_sah = ornament.Bvh(scene, row_major_transforms=True, builder="sah")
        r, st = renderer(kernel, bvh_sah if method in on_sah else None)
        if batched:
            st.spp_per_launch = streams
            st.sampler = _lib.SAMPLER_SOBOL if batched_sobol else _lib.SAMPLER_PCG
        cache = None
        t = 0.0
        if kernel != _lib.KERNEL_MEGA:
            if method == "light_sampling":
                cfg = {"train_shift": 0, "steps_per_frame": 0}
            elif batched:
                # training slots for 1/8 of the samples, filled at cache
                # vertices; one pass over the frame's training data (steps
                # capped by the slots)
                cfg = batched_cfg or {"train_shift": 3, "learning_rate": 5e-3, "steps_per_frame": 64}
            elif tuned:
                cfg = {"train_shift": 3, "learning_rate": 3e-3}
            else:
                cfg = cache_cfg or {"train_shift": 3}
            cache = ornament.RadianceCache(seed=1, **cfg)
            r.attach_cache(cache)
        if method.startswith("cached"):
            # warm-up training, then the accumulation restarts
            if batched:
                st.iterations = max(1, -(-batched_warmup_spp // streams))
            else:
                st.iterations = 32 if tuned else warmup
            r.set_state(st.to_struct())
            r.render()
            t += r.last_render_ms() / 1e3
            r.set_camera(scene.camera.to_struct())
        curve, n, chunk = [], 0, 16
        while True:
            st.iterations = chunk
            r.set_state(st.to_struct())
            r.render()
            t += r.last_render_ms() / 1e3
            n += chunk * (streams if batched else 1)
            e = r.relmse(ref)
            curve.append((t, n, e))
            if e <= target or t >= budget_s:
                break
            chunk = min(max(chunk + 1, chunk * 3 // 2), 1024)   # x1.5: finer readings near the target
        tt, reached = crossing_time(curve, target)
        out[method] = {"seconds": round(tt, 4), "reached": reached,
                       "samples_per_pixel": n, "final_relmse": curve[-1][2],
                       "tree": "SAH" if method in on_sah else "parity",
                       "curve": [[round(a, 4), b, float("%.4g" % c)] for a, b, c in curve]}
        r.close()
        if cache is not None:
            cache.close()
    for m in ("cached_batched", "cached_batched_wavefront"):
        if m in out:
            out[m]["streams"] = streams
    for m in ("plain_sah", "cached", "cached_tuned", "cached_batched", "cached_batched_wavefront", "light_sampling"):
        if m in out and "plain" in out:
            out[f"speedup_{m}_vs_plain"] = round(out["plain"]["seconds"] / out[m]["seconds"], 3)
    for m in ("cached_tuned", "cached_batched", "cached_batched_wavefront"):
        if m in out and "plain_sah" in out:
            out[f"speedup_{m}_vs_plain_same_tree"] = round(out["plain_sah"]["seconds"] / out[m]["seconds"], 3)
    if "speedup_cached_batched_vs_plain_same_tree" in out:
        v = out["speedup_cached_batched_vs_plain_same_tree"]
        out["target_5x_same_tree"] = ("met" if v >= 5.0 else f"not met ({v}x against the plain megakernel on "
                                      "the same SAH tree)")
    out["_ref"] = ref
    return out


def relmse_block(args):
    """The radiance-cache configuration's scene at its own resolution
    (--relmse-width x --relmse-height, default 1920x1080), and the closed
    room (a scene this project adds: long multi-bounce paths) at 640x360.
    With --workload large: the large scene (depth 16) at 960x540 instead —
    its 16k-sample FP64 oracle at 3840x2160 would take about an hour of GPU
    time at the plain megakernel's rate."""
    res = {"target": args.relmse_target, "metric": "GPU seconds to relMSE <= target vs FP64 oracle",
           "scenes": {}}
    if args.workload == "large":
        todo = (("large", 960, 540, 16),)
    else:
        todo = (("instanced", args.relmse_width, args.relmse_height, 8), ("closed-room", 640, 360, 8))
    for name, w, h, depth in todo:
        t0 = time.time()
        from zig_ornament_gb300 import _lib
        ck = _lib.KERNEL_CACHED_WAVEFRONT if args.cached_kernel == "wavefront" else _lib.KERNEL_CACHED
        res["scenes"][name] = time_to_relmse(name, w, h, args.relmse_target, args.relmse_ref_spp, args.relmse_budget,
                                             depth=depth, cached_kernel=ck)
        res["scenes"][name].pop("_ref")
        res["scenes"][name]["wall_s"] = round(time.time() - t0, 1)
    return res


def run_cached_frames(args):
    """A profiling workload: --frames radiance-cache frames (after 4 warm-up
    frames) of --scene at --width x --height; --batched for the cached +
    batched configuration."""
    from zig_ornament_gb300 import _lib, ornament
    scene = relmse_scene(args.scene, args.width, args.height)
    bvh = ornament.Bvh(scene, row_major_transforms=True, builder="sah" if args.batched else "reference")
    r = ornament.Renderer(bvh, 0)
    r.set_resolution(args.width, args.height)
    st = ornament.State()
    st.depth = args.depth
    st.kernel = _lib.KERNEL_CACHED_WAVEFRONT if args.cached_kernel == "wavefront" else _lib.KERNEL_CACHED
    cfg = {}
    if args.batched:
        st.spp_per_launch = 8
        st.sampler = _lib.SAMPLER_SOBOL
        cfg = {"train_shift": 3, "learning_rate": 5e-3, "steps_per_frame": 64}
    cache = ornament.RadianceCache(seed=1, **cfg)
    r.attach_cache(cache)
    r.set_state(st.to_struct())
    r.set_camera(scene.camera.to_struct())
    st.iterations = 4
    r.set_state(st.to_struct())
    r.render()
    st.iterations = args.frames
    r.set_state(st.to_struct())
    r.render()
    r.synchronize()
    print(json.dumps({"mode": "cached-frames", "scene": args.scene, "width": args.width, "height": args.height,
                      "batched": bool(args.batched), "samples_per_frame": args.width * args.height * max(
                          1, st.spp_per_launch), "frames": args.frames, "ms_per_frame": r.last_render_ms() / args.frames,
                      "cache": cache.stats()}), flush=True)
    r.attach_cache(None)
    r.close()
    cache.close()


def batch_measure(args, divisor=None):
    """The batched-rendering configuration: --batch-scenes independent
    instanced-mesh scenes (total BLAS triangles log-uniform 1k-2M, 1-1024
    instances, resolutions from {256^2, 640x360, 1280x720, 1920x1080}, 16-256
    samples per pixel, depth 8), one frame = spp/divisor passes of every
    scene (divisor 1: every scene's full sample count).  Sequential: each
    context's own orn_render (one megakernel launch per scene), summed device
    times; batched: orn_batch_render (one persistent launch replayed from a
    CUDA graph, launch shape from the autotuner), device time per frame."""
    from zig_ornament_gb300 import ornament, scenes
    divisor = divisor or args.batch_spp_divisor
    t0 = time.time()
    work = scenes.batch_scenes(count=args.batch_scenes, seed=2)
    ctxs, samples, nodes, rays = [], 0, 0, 0
    for sc, w, h, spp in work:
        bvh = ornament.Bvh(sc, row_major_transforms=True)
        r = ornament.Renderer(bvh, 0)
        r.set_resolution(w, h)
        st = ornament.State()
        st.depth = args.depth
        st.iterations = max(1, -(-spp // divisor))
        r.set_state(st.to_struct())
        r.set_camera(sc.camera.to_struct())
        ctxs.append(r)
        samples += w * h * st.iterations
        blob, keep = bvh.blob()
        nodes += blob.blas_nodes_len
        del keep
    setup_s = time.time() - t0
    # sequential: one render per context, each timed on its own stream
    for _ in range(args.warmup):
        for r in ctxs:
            r.render()
            r.synchronize()
    seq_ms = []
    for _ in range(args.steps):
        total = 0.0
        for r in ctxs:
            r.render()
            total += r.last_render_ms()
        seq_ms.append(total)
    # the work of one frame (exact counters, untimed)
    for r in ctxs:
        r.enable_counters(True)
        r.render()
        rays += r.counters()["rays"]
        r.enable_counters(False)
    batch = ornament.Batch(ctxs)
    t1 = time.time()
    cfg = batch.tune(args.tune_cache)
    tune_s = time.time() - t1
    for _ in range(args.warmup):
        batch.render()
    batch.synchronize()
    bat_ms = []
    with ClockSampler(0) as clocks:
        for _ in range(args.steps):
            batch.render()
            bat_ms.append(batch.last_render_ms())
    seq = samples / (np.mean(seq_ms) / 1e3) / 1e6
    bat = samples / (np.mean(bat_ms) / 1e3) / 1e6
    line = {"metric": "Msamples/s, batched scenes", "unit": "Msamples/s",
            "value": bat, "sequential": seq, "speedup": bat / seq,
            "rays_per_s": rays / samples * bat * 1e6,
            "ms_per_frame": {"batched": float(np.mean(bat_ms)), "sequential": float(np.mean(seq_ms))},
            "steps": args.steps, "warmup": args.warmup,
            "config": {"workload": f"{len(ctxs)} instanced-mesh scenes, total BLAS triangles log-uniform "
                                   "1k-2M, 1-1024 instances, resolutions 256^2..1920x1080, 16-256 spp, depth "
                                   f"{args.depth}; one frame = "
                                   + ("every scene's full sample count" if divisor == 1 else
                                      f"spp/{divisor} passes per scene"),
                       "pixels": int(sum(w * h for _, w, h, _ in work)), "samples_per_frame": int(samples),
                       "blas_nodes": int(nodes), "launch": cfg, "tune_seconds": round(tune_s, 2),
                       "setup_seconds": round(setup_s, 1)},
            "gpu_launches_per_frame": {"batched": 1, "sequential": len(ctxs)},
            "clocks": clocks.summary()}
    batch.close()
    for r in ctxs:
        r.close()
    return line


def run_batch(args):
    line = batch_measure(args)
    line["mode"] = "batch"
    line["batched"] = line["value"]
    print(json.dumps(line), flush=True)


def main():
    args = apply_workload_defaults(parse())
    if args.impl == "reference":
        run_reference(args)
    elif args.mode == "relmse":
        if int(os.environ.get("RANK", "0")) == 0:
            print(json.dumps({"mode": "relmse", "time_to_relmse": relmse_block(args)}), flush=True)
    elif args.mode == "batch":
        if int(os.environ.get("RANK", "0")) == 0:
            run_batch(args)
    elif args.mode == "cached-frames":
        if int(os.environ.get("RANK", "0")) == 0:
            run_cached_frames(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
