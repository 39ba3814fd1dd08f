"""ctypes binding of libornament_cuda (include/ornament_cuda.h).

The structures below are field-for-field copies of the C header; their sizes
are checked against the layouts of zig_ornament's src/gpu_structs.zig on
import.  Loading fails loudly when the library has not been built: there is
no fallback implementation.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libornament_cuda.so"

ORN_OK = 0
STATUS_NAMES = {
    0: "ORN_OK", 1: "ORN_ERR_INVALID_ARGUMENT", 2: "ORN_ERR_EMPTY_SCENE", 3: "ORN_ERR_OUT_OF_MEMORY",
    4: "ORN_ERR_CUDA", 5: "ORN_ERR_NO_DEVICE", 6: "ORN_ERR_BAD_SCENE", 7: "ORN_ERR_STACK_OVERFLOW",
    8: "ORN_ERR_BUFFER_TOO_SMALL", 9: "ORN_ERR_TIMEOUT", 10: "ORN_ERR_UNSUPPORTED", 11: "ORN_ERR_BAD_IMAGE",
}
NODE_INTERNAL, NODE_SPHERE, NODE_MESH, NODE_TRIANGLE = 0, 1, 2, 3
LAMBERTIAN, METAL, DIELECTRIC, DIFFUSE_LIGHT = 0, 1, 2, 3
NO_TEXTURE = 0xFFFFFFFF
TEXEL_RGBA8, TEXEL_RGBA16F = 0, 1
SEMANTICS_HIP, SEMANTICS_WGSL = 0, 1
KERNEL_MEGA, KERNEL_WAVEFRONT = 0, 1
COUNTER_COUNT = 10
NOALLOC_MAX_PIXELS = 131072
NOALLOC_MAX_DEPTH = 64
CACHE_INPUTS = 10
CACHE_OUTPUTS = 3
CACHE_PARAM_COUNT = 33792
KERNEL_CACHED = 2
KERNEL_CACHED_WAVEFRONT = 3
BATCH_MAX = 64
BVH_REFERENCE, BVH_SAH, BVH_LBVH = 0, 1, 2
TRIANGLE_MOLLER_TRUMBORE, TRIANGLE_WATERTIGHT = 0, 1
PIXEL_ORDER_COST, PIXEL_ORDER_RASTER = 0, 1
SAMPLER_PCG, SAMPLER_SOBOL = 0, 1
COUNTER_NAMES = ["samples", "rays", "visits", "internal", "sphere_leaf", "mesh_entry", "triangle",
                 "sphere_hits", "mesh_hits", "textured_hits"]

f3 = C.c_float * 3
f16 = C.c_float * 16


class BvhNode(C.Structure):
    _fields_ = [("left_aabb_min_or_v0", f3), ("left_or_custom_id", C.c_uint32),
                ("left_aabb_max_or_v1", f3), ("right_or_material_index", C.c_uint32),
                ("right_aabb_min_or_v2", f3), ("node_type", C.c_uint32),
                ("right_aabb_max_or_v3", f3), ("transform_id", C.c_uint32)]


class Material(C.Structure):
    _fields_ = [("albedo", f3), ("albedo_texture_index", C.c_uint32), ("fuzz", C.c_float),
                ("ior", C.c_float), ("type", C.c_uint32), ("_padding", C.c_uint32)]


class Camera(C.Structure):
    _fields_ = [("origin", f3), ("lens_radius", C.c_float),
                ("lower_left_corner", f3), ("_padding0", C.c_uint32),
                ("horizontal", f3), ("_padding1", C.c_uint32),
                ("vertical", f3), ("_padding2", C.c_uint32),
                ("u", f3), ("_padding3", C.c_uint32),
                ("v", f3), ("_padding4", C.c_uint32),
                ("w", f3), ("_padding5", C.c_uint32)]


class ConstantParams(C.Structure):
    _fields_ = [("camera", Camera), ("depth", C.c_uint32), ("width", C.c_uint32),
                ("height", C.c_uint32), ("flip_y", C.c_uint32), ("inverted_gamma", C.c_float),
                ("ray_cast_epsilon", C.c_float), ("textures_count", C.c_uint32),
                ("current_iteration", C.c_float)]


class Texture(C.Structure):
    _fields_ = [("data", C.c_void_p), ("width", C.c_uint32), ("height", C.c_uint32),
                ("bytes_per_row", C.c_uint32), ("format", C.c_uint32)]


class SceneBlob(C.Structure):
    _fields_ = [("tlas_nodes", C.c_void_p), ("tlas_nodes_len", C.c_uint32),
                ("blas_nodes", C.c_void_p), ("blas_nodes_len", C.c_uint32),
                ("normals", C.c_void_p), ("normals_len", C.c_uint32),
                ("normal_indices", C.c_void_p), ("normal_indices_len", C.c_uint32),
                ("uvs", C.c_void_p), ("uvs_len", C.c_uint32),
                ("uv_indices", C.c_void_p), ("uv_indices_len", C.c_uint32),
                ("transforms", C.c_void_p), ("transforms_len", C.c_uint32),
                ("materials", C.c_void_p), ("materials_len", C.c_uint32),
                ("textures", C.c_void_p), ("textures_len", C.c_uint32),
                ("scene_textures_count", C.c_uint32)]


class State(C.Structure):
    _fields_ = [("depth", C.c_uint32), ("flip_y", C.c_uint32), ("inverted_gamma", C.c_float),
                ("iterations", C.c_uint32), ("ray_cast_epsilon", C.c_float),
                ("semantics", C.c_uint32), ("kernel", C.c_uint32), ("spp_per_launch", C.c_uint32),
                ("triangle_test", C.c_uint32), ("pixel_order", C.c_uint32),
                ("sampler", C.c_uint32)]


class Ray(C.Structure):
    _fields_ = [("origin", f3), ("direction", f3)]


class Hit(C.Structure):
    _fields_ = [("hit", C.c_uint32), ("t", C.c_float), ("material_index", C.c_uint32),
                ("node_type", C.c_uint32), ("inverted_transform_id", C.c_uint32),
                ("tri_id", C.c_uint32), ("uv", C.c_float * 2)]


class MaterialDesc(C.Structure):
    _fields_ = [("albedo", f3), ("texture", C.c_uint32), ("fuzz", C.c_float), ("ior", C.c_float),
                ("type", C.c_uint32)]


class SphereDesc(C.Structure):
    _fields_ = [("transform", f16), ("aabb_min", f3), ("aabb_max", f3), ("material", C.c_uint32)]


class MeshDesc(C.Structure):
    _fields_ = [("vertices", C.c_void_p), ("vertices_len", C.c_uint32),
                ("vertex_indices", C.c_void_p), ("vertex_indices_len", C.c_uint32),
                ("normals", C.c_void_p), ("normals_len", C.c_uint32),
                ("normal_indices", C.c_void_p), ("normal_indices_len", C.c_uint32),
                ("uvs", C.c_void_p), ("uvs_len", C.c_uint32),
                ("uv_indices", C.c_void_p), ("uv_indices_len", C.c_uint32),
                ("transform", f16), ("aabb_min", f3), ("aabb_max", f3), ("material", C.c_uint32)]


class MeshInstanceDesc(C.Structure):
    _fields_ = [("mesh", C.c_uint32), ("transform", f16), ("aabb_min", f3), ("aabb_max", f3),
                ("material", C.c_uint32)]


class SceneDesc(C.Structure):
    _fields_ = [("spheres", C.c_void_p), ("spheres_len", C.c_uint32),
                ("meshes", C.c_void_p), ("meshes_len", C.c_uint32),
                ("mesh_instances", C.c_void_p), ("mesh_instances_len", C.c_uint32),
                ("materials", C.c_void_p), ("materials_len", C.c_uint32),
                ("textures", C.c_void_p), ("textures_len", C.c_uint32),
                ("seed", C.c_uint64), ("row_major_transforms", C.c_uint32), ("builder", C.c_uint32)]


# src/gpu_structs.zig layouts: BvhNode 64 B, Material 32 B, Camera 112 B, ConstantParams 144 B
assert C.sizeof(BvhNode) == 64 and C.sizeof(Material) == 32
assert C.sizeof(Camera) == 112 and C.sizeof(ConstantParams) == 144
assert C.sizeof(Ray) == 24 and C.sizeof(Hit) == 32

# name -> (restype, argtypes); every function declared in include/ornament_cuda.h
class CacheConfig(C.Structure):
    _fields_ = [("batch", C.c_uint32), ("steps_per_frame", C.c_uint32), ("train_shift", C.c_uint32),
                ("learning_rate", C.c_float), ("beta1", C.c_float), ("beta2", C.c_float),
                ("epsilon", C.c_float), ("reserved", C.c_uint32)]


class BatchConfig(C.Structure):
    _fields_ = [("block", C.c_uint32), ("blocks_per_sm", C.c_uint32), ("shade_threshold", C.c_uint32),
                ("tuned", C.c_uint32)]


class WaveConfig(C.Structure):
    _fields_ = [("shape", C.c_uint32), ("fetch", C.c_uint32), ("steps", C.c_uint32), ("tuned", C.c_uint32)]


_P = C.c_void_p
FUNCTIONS = {
    "orn_create": (C.c_int, [_P, C.c_int, C.POINTER(C.c_void_p)]),
    "orn_destroy": (C.c_int, [_P]),
    "orn_set_state": (C.c_int, [_P, C.POINTER(State)]),
    "orn_get_state": (C.c_int, [_P, C.POINTER(State)]),
    "orn_set_camera": (C.c_int, [_P, C.POINTER(Camera)]),
    "orn_set_resolution": (C.c_int, [_P, C.c_uint32, C.c_uint32]),
    "orn_get_resolution": (C.c_int, [_P, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
    "orn_render": (C.c_int, [_P]),
    "orn_synchronize": (C.c_int, [_P]),
    "orn_get_framebuffer": (C.c_int, [_P, _P, C.c_size_t]),
    "orn_get_accumulation": (C.c_int, [_P, _P, C.c_size_t]),
    "orn_get_progress": (C.c_int, [_P, _P, _P, C.c_size_t, C.POINTER(C.c_float)]),
    "orn_set_progress": (C.c_int, [_P, _P, _P, C.c_size_t, C.c_float]),
    "orn_peek_constant_params": (C.c_int, [_P, C.POINTER(ConstantParams)]),
    "orn_trace_rays": (C.c_int, [_P, _P, C.c_size_t, _P, _P]),
    "orn_enable_counters": (C.c_int, [_P, C.c_int]),
    "orn_get_counters": (C.c_int, [_P, C.POINTER(C.c_uint64), C.c_size_t]),
    "orn_last_render_ms": (C.c_int, [_P, C.POINTER(C.c_float)]),
    "orn_get_stream": (C.c_int, [_P, C.POINTER(C.c_void_p)]),
    "orn_launch_count": (C.c_int, [_P, C.POINTER(C.c_uint64)]),
    "orn_render_noalloc": (C.c_int, [_P, C.POINTER(ConstantParams), C.c_uint32, _P, _P, _P, _P]),
    "orn_render_f64": (C.c_int, [_P, C.c_uint32, _P, C.c_size_t]),
    "orn_tc_selftest": (C.c_int, [C.c_uint32, C.c_uint32, C.c_int, C.c_int, _P, _P, _P]),
    "orn_relmse": (C.c_int, [_P, _P, C.c_size_t, C.POINTER(C.c_double), C.POINTER(C.c_uint64)]),
    "orn_cache_default_config": (C.c_int, [C.POINTER(CacheConfig)]),
    "orn_cache_create": (C.c_int, [C.c_int, C.c_uint64, C.POINTER(CacheConfig), C.POINTER(C.c_void_p)]),
    "orn_cache_destroy": (C.c_int, [_P]),
    "orn_cache_set_config": (C.c_int, [_P, C.POINTER(CacheConfig)]),
    "orn_cache_get_params": (C.c_int, [_P, _P, C.c_size_t]),
    "orn_cache_set_params": (C.c_int, [_P, _P, C.c_size_t]),
    "orn_cache_infer": (C.c_int, [_P, _P, C.c_size_t, _P]),
    "orn_cache_gradients": (C.c_int, [_P, _P, _P, C.c_size_t, _P, C.POINTER(C.c_float)]),
    "orn_cache_train": (C.c_int, [_P, _P, _P, C.c_size_t, C.POINTER(C.c_float)]),
    "orn_cache_stats": (C.c_int, [_P, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.POINTER(C.c_float)]),
    "orn_cache_last_error": (C.c_char_p, [_P]),
    "orn_attach_cache": (C.c_int, [_P, _P]),
    "orn_get_device": (C.c_int, [_P, C.POINTER(C.c_int)]),
    "orn_batch_create": (C.c_int, [_P, C.c_uint32, C.POINTER(C.c_void_p)]),
    "orn_batch_destroy": (C.c_int, [_P]),
    "orn_batch_render": (C.c_int, [_P]),
    "orn_batch_synchronize": (C.c_int, [_P]),
    "orn_batch_last_render_ms": (C.c_int, [_P, C.POINTER(C.c_float)]),
    "orn_batch_get_config": (C.c_int, [_P, C.POINTER(BatchConfig)]),
    "orn_batch_set_config": (C.c_int, [_P, C.POINTER(BatchConfig)]),
    "orn_batch_tune": (C.c_int, [_P, C.c_char_p, C.POINTER(BatchConfig)]),
    "orn_wave_get_config": (C.c_int, [_P, C.POINTER(WaveConfig)]),
    "orn_wave_set_config": (C.c_int, [_P, C.POINTER(WaveConfig)]),
    "orn_wave_tune": (C.c_int, [_P, C.c_char_p, C.POINTER(WaveConfig)]),
    "orn_batch_last_error": (C.c_char_p, [_P]),
    "orn_last_error": (C.c_char_p, [_P]),
    "orn_status_string": (C.c_char_p, [C.c_int]),
    "orn_abi_version": (C.c_uint32, []),
    "orn_bvh_build": (C.c_int, [_P, C.POINTER(C.c_void_p)]),
    "orn_bvh_get_blob": (C.c_int, [_P, C.POINTER(SceneBlob)]),
    "orn_bvh_free": (C.c_int, [_P]),
    "orn_jpeg_info": (C.c_int, [_P, C.c_size_t, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                C.POINTER(C.c_uint32)]),
    "orn_jpeg_decode": (C.c_int, [_P, C.c_size_t, C.c_int, C.c_uint32, _P, C.c_size_t]),
    "orn_jpeg_coefficients": (C.c_int, [_P, C.c_size_t, C.c_uint32, _P, C.c_size_t, C.POINTER(C.c_uint32),
                                        C.POINTER(C.c_uint32), _P]),
    "orn_jpeg_last_error": (C.c_char_p, []),
    "orn_qmc_points": (C.c_int, [C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, _P]),
}

_lib = None


class OrnamentError(RuntimeError):
    def __init__(self, status: int, message: str):
        self.status = status
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")


def load(path: os.PathLike | str | None = None) -> C.CDLL:
    """Loads libornament_cuda.so (built in-tree by zig_ornament_gb300.build)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise OrnamentError(-1, f"{p} is missing: build it with "
                                "`python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(str(p))
    for name, (res, args) in FUNCTIONS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.orn_abi_version() != 1:
        raise OrnamentError(-1, "libornament_cuda ABI version mismatch")
    if path is None:
        _lib = lib
    return lib


def check(status: int, ctx=None) -> None:
    if status != ORN_OK:
        lib = load()
        msg = lib.orn_last_error(ctx).decode() if ctx else lib.orn_status_string(status).decode()
        raise OrnamentError(status, msg or lib.orn_status_string(status).decode())
