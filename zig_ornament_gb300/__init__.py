"""zig_ornament_gb300 — a GB300 (sm_103a) path-tracing backend for the
zig_ornament scene model.

The compute path is libornament_cuda.so (hand-written CUDA, C ABI in
include/ornament_cuda.h); this package holds its build script, the ctypes
binding and a Python mirror of ornament.zig's Scene / Camera / State /
PathTracer surface.
"""
from .ornament import (Aabb, Bvh, Camera, Material, Mesh, MeshInstance, PathTracer, Resolution, Scene,
                       Sphere, State, Texture)

__all__ = ["Aabb", "Bvh", "Camera", "Material", "Mesh", "MeshInstance", "PathTracer", "Resolution",
           "Scene", "Sphere", "State", "Texture"]
