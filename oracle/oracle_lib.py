"""ctypes wrappers of the CPU oracles (test infrastructure only).

Oracle    — oracle/oracle.cpp, the restatement (always available after
            build_oracle()).
Reference — the reference's own HIP kernels compiled for the host
            (oracle/_ref, available where the zig_ornament sources are).
Both take a Bvh (zig_ornament_gb300.ornament.Bvh or Bvh.from_arrays) and
orn_constant_params, and return numpy arrays.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build_oracle as bo

_P = C.c_void_p


def _ptr(a):
    return a.ctypes.data if a is not None and a.size else None


class Oracle:
    def __init__(self, path=None):
        path = path or bo.build_oracle()
        self.lib = C.CDLL(str(path))
        self.lib.oracle_trace_rays.restype = C.c_int
        self.lib.oracle_trace_rays.argtypes = [_P, C.c_float, _P, C.c_size_t, _P, _P, C.c_int]
        self.lib.oracle_render.restype = C.c_int
        self.lib.oracle_render.argtypes = [_P, _P, C.c_uint32, C.c_float, C.c_int, C.c_int, _P, _P, _P, _P,
                                           C.c_uint32, C.c_uint32, C.c_uint32, C.c_int, _P]
        for fn in ("oracle_pm_eval", "oracle_libm_eval"):
            getattr(self.lib, fn).restype = None
            getattr(self.lib, fn).argtypes = [C.c_int, _P, _P, _P, _P, C.c_size_t]

    def trace_rays(self, bvh, rays, eps=0.001, threads=0):
        from zig_ornament_gb300.ornament import HIT_DTYPE
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 6)
        hits = np.zeros(len(rays), dtype=HIT_DTYPE)
        visits = np.zeros(len(rays), dtype=np.uint32)
        blob, keep = bvh.blob()
        st = self.lib.oracle_trace_rays(C.byref(blob), eps, _ptr(rays), len(rays), _ptr(hits), _ptr(visits), threads)
        if st != 0:
            raise RuntimeError(f"oracle_trace_rays failed with status {st}")
        return hits, visits

    def render(self, bvh, cp, spp, ci_start=1.0, acc=None, rng=None, semantics=0, portable_math=True,
               acc64=None, pixel_range=None, pixel_stride=1, threads=0, counters=False):
        """Returns (acc, rng, fb, counters).  acc/rng default to a fresh
        target (zeros, RNG seeded with the pixel index)."""
        n = cp.width * cp.height
        acc = np.zeros((n, 4), np.float32) if acc is None else np.ascontiguousarray(acc, np.float32).copy()
        rng = np.arange(n, dtype=np.uint32) if rng is None else np.ascontiguousarray(rng, np.uint32).copy()
        fb = np.zeros((n, 4), np.float32)
        cnt = np.zeros(10, np.uint64) if counters else None
        lo, hi = pixel_range if pixel_range else (0, n)
        blob, keep = bvh.blob()
        st = self.lib.oracle_render(C.byref(blob), C.byref(cp), spp, ci_start, semantics, 1 if portable_math else 0,
                                    _ptr(acc), _ptr(rng), _ptr(fb), _ptr(acc64), lo, hi, pixel_stride, threads,
                                    _ptr(cnt))
        if st != 0:
            raise RuntimeError(f"oracle_render failed with status {st}")
        return acc, rng, fb, cnt

    def pm_eval(self, fn, a, b=None, libm=False):
        a = np.ascontiguousarray(a, np.float32)
        b = np.ascontiguousarray(b if b is not None else np.zeros_like(a), np.float32)
        out = np.zeros_like(a)
        out2 = np.zeros_like(a)
        f = self.lib.oracle_libm_eval if libm else self.lib.oracle_pm_eval
        f({"pow": 0, "acos": 1, "atan2": 2, "sincos": 3}[fn], _ptr(a), _ptr(b), _ptr(out), _ptr(out2), len(a))
        return (out, out2) if fn == "sincos" else out


class Reference:
    """The reference's HIP kernels compiled for the host."""

    def __init__(self, portable_math=False):
        paths = bo.build_ref()
        if paths is None:
            raise FileNotFoundError("zig_ornament sources not found (set ORN_REFERENCE_DIR)")
        self.lib = C.CDLL(str(paths[1] if portable_math else paths[0]))
        self.lib.ref_render.restype = C.c_int
        self.lib.ref_render.argtypes = [_P, _P, C.c_uint32, C.c_float, _P, _P, _P, C.c_int]
        self.lib.ref_trace_rays.restype = C.c_int
        self.lib.ref_trace_rays.argtypes = [_P, C.c_float, _P, C.c_size_t, _P, C.c_int]
        self.lib.ref_struct_sizes.restype = C.c_int
        self.lib.ref_struct_sizes.argtypes = [_P, C.c_int]

    def struct_sizes(self):
        out = np.zeros(5, np.uint32)
        self.lib.ref_struct_sizes(_ptr(out), 5)
        return dict(zip(["BvhNode", "Material", "ConstantParams", "Camera", "float4x4"], out.tolist()))

    def render(self, bvh, cp, spp, ci_start=1.0, acc=None, rng=None, threads=0):
        n = cp.width * cp.height
        acc = np.zeros((n, 4), np.float32) if acc is None else np.ascontiguousarray(acc, np.float32).copy()
        rng = np.arange(n, dtype=np.uint32) if rng is None else np.ascontiguousarray(rng, np.uint32).copy()
        fb = np.zeros((n, 4), np.float32)
        blob, keep = bvh.blob()
        st = self.lib.ref_render(C.byref(blob), C.byref(cp), spp, ci_start, _ptr(acc), _ptr(rng), _ptr(fb), threads)
        if st != 0:
            raise RuntimeError(f"ref_render failed with status {st}")
        return acc, rng, fb

    def trace_rays(self, bvh, rays, eps=0.001, threads=0):
        from zig_ornament_gb300.ornament import HIT_DTYPE
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 6)
        hits = np.zeros(len(rays), dtype=HIT_DTYPE)
        blob, keep = bvh.blob()
        st = self.lib.ref_trace_rays(C.byref(blob), eps, _ptr(rays), len(rays), _ptr(hits), threads)
        if st != 0:
            raise RuntimeError(f"ref_trace_rays failed with status {st}")
        return hits


def reference_available() -> bool:
    return bo.reference_available()


def make_params(camera, width, height, depth=10, flip_y=False, gamma=1.0, eps=0.001, textures_count=0,
                current_iteration=1.0):
    """orn_constant_params from an ornament Camera (ConstantParams.from,
    src/gpu_structs.zig:73-85)."""
    from zig_ornament_gb300 import _lib
    import numpy as _np
    cp = _lib.ConstantParams()
    cp.camera = camera.to_struct() if hasattr(camera, "to_struct") else camera
    cp.depth, cp.width, cp.height = depth, width, height
    cp.flip_y = 1 if flip_y else 0
    cp.inverted_gamma = float(_np.float32(1.0) / _np.float32(gamma))
    cp.ray_cast_epsilon = eps
    cp.textures_count = textures_count
    cp.current_iteration = current_iteration
    return cp
