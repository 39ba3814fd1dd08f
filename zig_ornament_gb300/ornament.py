"""Python mirror of zig_ornament's public surface (src/ornament.zig:1-19).

The names, argument meanings and defaults follow the Zig sources so that a
driver written against ornament.zig reads the same here:

  Scene         src/scene.zig:13-380  (lambertian/metal/dielectric/diffuseLight,
                createSphere/createSphereMesh/createPlaneMesh/createMesh/
                createMeshInstance/createTexture, attach*)
  Camera        src/camera.zig:4-114  (init, setAspectRatio, setLookAt, dirty)
  State         src/state.zig:3-80
  Aabb          src/aabb.zig:3-45
  Bvh           src/bvh.zig:33-90     (built by libornament_cuda's orn_bvh_build)
  PathTracer    src/hip_backend/path_tracer.zig:12-236 (init, deinit,
                setResolution, render, getFrameBuffer, public scene/state)

Matrices follow zmath: row vectors, v' = v · M, translation in row 3,
``mul(a, b)`` applies ``a`` first.  All arithmetic is float32.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field
from typing import List, Optional, Sequence, Union

import numpy as np

from . import _lib

F32 = np.float32

# ---------------------------------------------------------------- zmath subset


def f32x4(x, y, z, w) -> np.ndarray:
    return np.array([x, y, z, w], dtype=F32)


def identity() -> np.ndarray:
    return np.eye(4, dtype=F32)


def scaling(x, y, z) -> np.ndarray:
    m = identity()
    m[0, 0], m[1, 1], m[2, 2] = x, y, z
    return m


def scalingV(v) -> np.ndarray:
    return scaling(v[0], v[1], v[2])


def translation(x, y, z) -> np.ndarray:
    m = identity()
    m[3, 0], m[3, 1], m[3, 2] = x, y, z
    return m


def translationV(v) -> np.ndarray:
    return translation(v[0], v[1], v[2])


def rotationX(a) -> np.ndarray:
    c, s = F32(math.cos(a)), F32(math.sin(a))
    return np.array([[1, 0, 0, 0], [0, c, s, 0], [0, -s, c, 0], [0, 0, 0, 1]], dtype=F32)


def rotationY(a) -> np.ndarray:
    c, s = F32(math.cos(a)), F32(math.sin(a))
    return np.array([[c, 0, -s, 0], [0, 1, 0, 0], [s, 0, c, 0], [0, 0, 0, 1]], dtype=F32)


def rotationZ(a) -> np.ndarray:
    c, s = F32(math.cos(a)), F32(math.sin(a))
    return np.array([[c, s, 0, 0], [-s, c, 0, 0], [0, 0, 1, 0], [0, 0, 0, 1]], dtype=F32)


def matFromQuat(q) -> np.ndarray:
    x, y, z, w = (F32(v) for v in q)
    return np.array([
        [1 - 2 * (y * y + z * z), 2 * (x * y + z * w), 2 * (x * z - y * w), 0],
        [2 * (x * y - z * w), 1 - 2 * (x * x + z * z), 2 * (y * z + x * w), 0],
        [2 * (x * z + y * w), 2 * (y * z - x * w), 1 - 2 * (x * x + y * y), 0],
        [0, 0, 0, 1]], dtype=F32)


def mul(a, b) -> np.ndarray:
    return np.asarray(a, dtype=F32) @ np.asarray(b, dtype=F32)


def dot3(a, b) -> F32:
    return F32(a[0] * b[0] + a[1] * b[1] + a[2] * b[2])


def cross3(a, b) -> np.ndarray:
    return f32x4(a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0], 0.0)


def length3(a) -> F32:
    return F32(math.sqrt(float(dot3(a, a))))


def normalize3(a) -> np.ndarray:
    v = np.asarray(a, dtype=F32).copy()
    v[:3] = v[:3] / length3(v)
    return v


unit_x = f32x4(1, 0, 0, 0)
unit_y = f32x4(0, 1, 0, 0)
unit_z = f32x4(0, 0, 1, 0)


def rotationBetweenVectors(a, b) -> np.ndarray:
    """src/math.zig:13-41."""
    k_cos_theta = float(dot3(a, b))
    if abs(k_cos_theta - 1.0) <= 1e-7:
        return identity()
    k = math.sqrt(float(dot3(a, a)) * float(dot3(b, b)))
    if abs(k_cos_theta / k + 1.0) <= 1e-7:
        orthogonal = cross3(a, unit_x)
        if abs(float(dot3(orthogonal, orthogonal))) <= 1e-7:
            orthogonal = cross3(a, unit_y)
        orthogonal = normalize3(orthogonal)
        return matFromQuat((orthogonal[0], orthogonal[1], orthogonal[2], 0.0))
    v = cross3(a, b)
    q = np.array([v[0], v[1], v[2], k + k_cos_theta], dtype=F32)
    q = q / F32(math.sqrt(float(np.dot(q, q))))
    return matFromQuat(q)


def getSphereTexCoord(p) -> np.ndarray:
    """src/math.zig:43-47."""
    theta = math.acos(-float(p[1]))
    phi = math.atan2(-float(p[2]), float(p[0])) + math.pi
    return np.array([phi / (2.0 * math.pi), theta / math.pi], dtype=F32)


# ------------------------------------------------------------------ scene model


@dataclass
class Aabb:
    """src/aabb.zig:3-45."""
    min: np.ndarray
    max: np.ndarray

    @staticmethod
    def transform(m, aabb: "Aabb") -> "Aabb":
        lo, hi = aabb.min, aabb.max
        corners = np.array([[x, y, z, 1.0] for x in (lo[0], hi[0]) for y in (lo[1], hi[1]) for z in (lo[2], hi[2])],
                           dtype=F32)
        p = corners @ np.asarray(m, dtype=F32)
        return Aabb(np.append(p[:, :3].min(axis=0), F32(1)).astype(F32),
                    np.append(p[:, :3].max(axis=0), F32(1)).astype(F32))


@dataclass(eq=False)
class Texture:
    """src/texture.zig:3-45.  RGBA only (num_components = 4); 1 byte per
    component is RGBA8 unorm, 2 bytes per component is RGBA16F (is_hdr)."""
    data: np.ndarray
    width: int
    height: int
    num_components: int = 4
    bytes_per_component: int = 1
    is_hdr: bool = False
    gamma: float = 1.0
    texture_id: Optional[int] = None

    @property
    def bytes_per_row(self) -> int:
        return self.width * self.num_components * self.bytes_per_component


Color = Union[Sequence[float], np.ndarray, Texture]


@dataclass(eq=False)
class Material:
    """src/material.zig:11-17."""
    albedo: Color
    fuzz: float = 0.0
    ior: float = 0.0
    type: int = _lib.LAMBERTIAN
    material_index: Optional[int] = None


@dataclass(eq=False)
class Sphere:
    material: Material
    transform: np.ndarray
    aabb: Aabb


@dataclass(eq=False)
class Mesh:
    vertices: np.ndarray          # (n, 4) float32
    vertex_indices: np.ndarray    # uint32
    normals: np.ndarray           # (n, 4) float32
    normal_indices: np.ndarray
    uvs: np.ndarray               # (n, 2) float32
    uv_indices: np.ndarray
    transform: np.ndarray
    material: Material
    aabb: Aabb
    not_transformed_aabb: Aabb
    bvh_id: Optional[int] = None


@dataclass(eq=False)
class MeshInstance:
    mesh: Mesh
    material: Material
    transform: np.ndarray
    aabb: Aabb


class Camera:
    """src/camera.zig:4-114."""

    def __init__(self, lookfrom, lookat, vup, aspect_ratio, vfov, aperture, focus_dist):
        self.init(lookfrom, lookat, vup, aspect_ratio, vfov, aperture, focus_dist)

    def init(self, lookfrom, lookat, vup, aspect_ratio, vfov, aperture, focus_dist):
        lookfrom, lookat, vup = (np.asarray(v, dtype=F32) for v in (lookfrom, lookat, vup))
        theta = F32(math.radians(vfov))
        h = F32(math.tan(theta / F32(2.0)))
        viewport_height = F32(2.0) * h
        viewport_width = F32(aspect_ratio) * viewport_height
        w = normalize3(lookfrom - lookat)
        u = normalize3(cross3(vup, w))
        v = cross3(w, u)
        fd = F32(focus_dist)
        self.origin = lookfrom
        self.horizontal = (fd * viewport_width) * u
        self.vertical = (fd * viewport_height) * v
        self.lower_left_corner = self.origin - self.horizontal / F32(2.0) - self.vertical / F32(2.0) - fd * w
        self.u, self.v, self.w = u, v, w
        self.lens_radius = F32(aperture) / F32(2.0)
        self.vfov, self.focus_dist, self.aspect_ratio = float(vfov), float(focus_dist), float(aspect_ratio)
        self.lookfrom, self.lookat, self.vup = lookfrom, lookat, vup
        self.dirty = True

    def setAspectRatio(self, aspect_ratio):
        self.init(self.lookfrom, self.lookat, self.vup, aspect_ratio, self.vfov, 2.0 * float(self.lens_radius),
                  self.focus_dist)

    def getAspectRatio(self):
        return self.aspect_ratio

    def getLookFrom(self):
        return self.lookfrom

    def getLookAt(self):
        return self.lookat

    def getVUp(self):
        return self.vup

    def setLookAt(self, lookfrom, lookat, vup):
        self.init(lookfrom, lookat, vup, self.aspect_ratio, self.vfov, 2.0 * float(self.lens_radius),
                  self.focus_dist)

    def to_struct(self) -> _lib.Camera:
        c = _lib.Camera()
        for name in ("origin", "lower_left_corner", "horizontal", "vertical", "u", "v", "w"):
            getattr(c, name)[:] = [float(x) for x in getattr(self, name)[:3]]
        c.lens_radius = float(self.lens_radius)
        return c


@dataclass
class Resolution:
    width: int
    height: int

    def pixel_count(self) -> int:
        return self.width * self.height


class State:
    """src/state.zig:3-80 plus the backend switches of this library
    (semantics, kernel, spp_per_launch)."""

    def __init__(self):
        self.resolution = Resolution(500, 500)
        self.depth = 10
        self.flip_y = False
        self.inverted_gamma = 1.0
        self.iterations = 1
        self.ray_cast_epsilon = 0.001
        self.current_iteration = 0.0
        self.semantics = _lib.SEMANTICS_HIP
        self.kernel = _lib.KERNEL_MEGA
        self.spp_per_launch = 0
        self.triangle_test = _lib.TRIANGLE_MOLLER_TRUMBORE
        self.pixel_order = _lib.PIXEL_ORDER_COST
        self.sampler = _lib.SAMPLER_PCG

    def setFlipY(self, v): self.flip_y = bool(v)
    def getFlipY(self): return self.flip_y
    def setGamma(self, g): self.inverted_gamma = float(F32(1.0) / F32(g))
    def getGamma(self): return 1.0 / self.inverted_gamma
    def setDepth(self, d): self.depth = int(d)
    def getDepth(self): return self.depth
    def setIterations(self, n): self.iterations = int(n)
    def getIterations(self): return self.iterations
    def setResolution(self, r): self.resolution = r
    def getResolution(self): return self.resolution
    def setRayCastEpsilon(self, e): self.ray_cast_epsilon = float(e)
    def getRayCastEpsilon(self): return self.ray_cast_epsilon
    def nextIteration(self): self.current_iteration += 1.0
    def reset(self): self.current_iteration = 0.0

    def to_struct(self) -> _lib.State:
        s = _lib.State()
        s.depth = self.depth
        s.flip_y = 1 if self.flip_y else 0
        s.inverted_gamma = self.inverted_gamma
        s.iterations = self.iterations
        s.ray_cast_epsilon = self.ray_cast_epsilon
        s.semantics = self.semantics
        s.kernel = self.kernel
        s.spp_per_launch = self.spp_per_launch
        s.triangle_test = self.triangle_test
        s.pixel_order = self.pixel_order
        s.sampler = self.sampler
        return s


def _vec4(v) -> np.ndarray:
    a = np.zeros(4, dtype=F32)
    a[:len(v)] = v
    return a


class Scene:
    """src/scene.zig:13-380."""

    def __init__(self):
        self.camera = Camera(f32x4(1, 1, 1, 1), f32x4(0, 0, 0, 1), f32x4(0, 1, 0, 0), 1.0, 40.0, 0.0, 10.0)
        self.spheres: List[Sphere] = []
        self.meshes: List[Mesh] = []
        self.mesh_instances: List[MeshInstance] = []
        self.materials: List[Material] = []
        self.textures: List[Texture] = []
        self.attached_spheres: List[Sphere] = []
        self.attached_meshes: List[Mesh] = []
        self.attached_mesh_instances: List[MeshInstance] = []

    # materials (src/scene.zig:64-118)
    def _material(self, m: Material) -> Material:
        self.materials.append(m)
        return m

    def lambertian(self, albedo: Color) -> Material:
        return self._material(Material(albedo=albedo, type=_lib.LAMBERTIAN))

    def metal(self, albedo: Color, fuzz: float) -> Material:
        return self._material(Material(albedo=albedo, fuzz=fuzz, type=_lib.METAL))

    def dielectric(self, ior: float) -> Material:
        return self._material(Material(albedo=(0.0, 0.0, 0.0), ior=ior, type=_lib.DIELECTRIC))

    def diffuseLight(self, albedo: Color) -> Material:
        return self._material(Material(albedo=albedo, type=_lib.DIFFUSE_LIGHT))

    # shapes
    def createSphere(self, center, radius: float, material: Material) -> Sphere:
        """src/scene.zig:124-134: transform = scaling(r) · translation(c)."""
        c = _vec4(center)
        r = F32(radius)
        radius_v = np.array([r, r, r, 0], dtype=F32)
        s = Sphere(material=material, transform=mul(scaling(r, r, r), translationV(c)),
                   aabb=Aabb(c - radius_v, c + radius_v))
        self.spheres.append(s)
        return s

    def createSphereMesh(self, center, radius: float, material: Material) -> Mesh:
        """src/scene.zig:140-233: UV sphere, 60 x 30 segments."""
        h_segments, v_segments = 60, 30
        vertices, normals, uvs, indices = [f32x4(0, 1, 0, 1)], [f32x4(0, 1, 0, 0)], [], []
        uvs.append(getSphereTexCoord(normals[-1]))
        for v in range(1, v_segments):
            theta = F32(v) / F32(v_segments) * F32(math.pi)
            sin_theta = F32(math.sin(theta))
            for h in range(h_segments):
                phi = F32(h) / F32(h_segments) * F32(math.pi) * F32(2.0)
                x = sin_theta * F32(math.sin(phi))
                z = sin_theta * F32(math.cos(phi))
                y = F32(math.cos(theta))
                vertices.append(f32x4(x, y, z, 1))
                normals.append(normalize3(f32x4(x, y, z, 0)))
                uvs.append(getSphereTexCoord(normals[-1]))
                if v == 1:
                    indices += [0, h + 1, h + 2 if h < h_segments - 1 else 1]
                else:
                    i = h + (v - 1) * h_segments + 1
                    j = i - h_segments
                    k = j + 1 if h < h_segments - 1 else j - (h_segments - 1)
                    l = i + 1 if h < h_segments - 1 else i - (h_segments - 1)
                    indices += [j, i, k, k, i, l]
        vertices.append(f32x4(0, -1, 0, 1))
        normals.append(f32x4(0, -1, 0, 0))
        uvs.append(getSphereTexCoord(normals[-1]))
        end = len(vertices) - 1
        for h in range(h_segments):
            i = end - h_segments + h
            indices += [i, end, i + 1 if h < h_segments - 1 else end - h_segments]
        transform = mul(scaling(radius, radius, radius), translationV(_vec4(center)))
        idx = np.array(indices, dtype=np.uint32)
        return self.createMesh(np.array(vertices), idx, np.array(normals), idx, np.array(uvs), idx,
                               transform, material)

    def createPlaneMesh(self, center, side1_length, side2_length, normal, material: Material) -> Mesh:
        """src/scene.zig:235-261."""
        vertices = np.array([[-0.5, 0, -0.5, 1], [-0.5, 0, 0.5, 1], [0.5, 0, 0.5, 1], [0.5, 0, -0.5, 1]], dtype=F32)
        indices = np.array([3, 1, 0, 2, 1, 3], dtype=np.uint32)
        normals = np.array([unit_y] * 4, dtype=F32)
        rotation = rotationBetweenVectors(_vec4(normal), unit_y)
        transform = mul(mul(scaling(side1_length, 1.0, side2_length), rotation), translationV(_vec4(center)))
        return self.createMesh(vertices, indices, normals, indices, np.zeros((0, 2), F32),
                               np.zeros(0, np.uint32), transform, material)

    def createMesh(self, vertices, vertex_indices, normals, normal_indices, uvs, uv_indices,
                   transform, material: Material) -> Mesh:
        """src/scene.zig:263-316.  Empty uvs become (0.5, 0.5) per vertex with
        uv_indices = vertex_indices."""
        vertices = np.ascontiguousarray(vertices, dtype=F32).reshape(-1, 4)
        vertex_indices = np.ascontiguousarray(vertex_indices, dtype=np.uint32).reshape(-1)
        normals = np.ascontiguousarray(normals, dtype=F32).reshape(-1, 4)
        normal_indices = np.ascontiguousarray(normal_indices, dtype=np.uint32).reshape(-1)
        uvs = np.ascontiguousarray(uvs, dtype=F32).reshape(-1, 2)
        uv_indices = np.ascontiguousarray(uv_indices, dtype=np.uint32).reshape(-1)
        ntri = len(vertex_indices) // 3
        tri = vertices[vertex_indices[:ntri * 3]].reshape(ntri, 3, 4) if ntri else np.zeros((0, 3, 4), F32)
        if ntri:
            mn = np.append(tri[:, :, :3].min(axis=(0, 1)), F32(1)).astype(F32)
            mx = np.append(tri[:, :, :3].max(axis=(0, 1)), F32(1)).astype(F32)
        else:
            mn = f32x4(np.inf, np.inf, np.inf, 1)
            mx = f32x4(-np.inf, -np.inf, -np.inf, 1)
        not_transformed = Aabb(mn, mx)
        if len(uvs) == 0:
            uvs = np.full((len(vertices), 2), 0.5, dtype=F32)
            uv_indices = vertex_indices.copy()
        m = Mesh(vertices=vertices, vertex_indices=vertex_indices, normals=normals,
                 normal_indices=normal_indices, uvs=uvs, uv_indices=uv_indices,
                 transform=np.asarray(transform, dtype=F32), material=material,
                 aabb=Aabb.transform(transform, not_transformed) if ntri else not_transformed,
                 not_transformed_aabb=not_transformed)
        self.meshes.append(m)
        return m

    def createMeshInstance(self, mesh: Mesh, transform, material: Material) -> MeshInstance:
        """src/scene.zig:323-333."""
        mi = MeshInstance(mesh=mesh, material=material, transform=np.asarray(transform, dtype=F32),
                          aabb=Aabb.transform(transform, mesh.not_transformed_aabb))
        self.mesh_instances.append(mi)
        return mi

    def createTexture(self, data, width, height, num_components=4, bytes_per_component=1,
                      is_hdr=False, gamma=1.0) -> Texture:
        """src/scene.zig:339-351."""
        if num_components != 4:
            raise ValueError("textures are RGBA (num_components = 4)")
        dtype = np.uint8 if bytes_per_component == 1 else np.float16
        arr = np.ascontiguousarray(data, dtype=dtype).reshape(height, width, 4)
        t = Texture(arr, int(width), int(height), 4, int(bytes_per_component), bool(is_hdr), float(gamma))
        self.textures.append(t)
        return t

    def attachSphere(self, s): self.attached_spheres.append(s)
    def attachMesh(self, m): self.attached_meshes.append(m)
    def attachMeshInstance(self, mi): self.attached_mesh_instances.append(mi)


# ---------------------------------------------------------------- BVH builder

NODE_DTYPE = np.dtype([("left_aabb_min_or_v0", F32, 3), ("left_or_custom_id", np.uint32),
                       ("left_aabb_max_or_v1", F32, 3), ("right_or_material_index", np.uint32),
                       ("right_aabb_min_or_v2", F32, 3), ("node_type", np.uint32),
                       ("right_aabb_max_or_v3", F32, 3), ("transform_id", np.uint32)])
MATERIAL_DTYPE = np.dtype([("albedo", F32, 3), ("albedo_texture_index", np.uint32), ("fuzz", F32),
                           ("ior", F32), ("type", np.uint32), ("_padding", np.uint32)])
assert NODE_DTYPE.itemsize == 64 and MATERIAL_DTYPE.itemsize == 32


def _ptr(a: np.ndarray):
    return a.ctypes.data if a.size else None


class Bvh:
    """Bvh.init (src/bvh.zig:33-78) through orn_bvh_build.

    The flat arrays are copied into numpy (``tlas_nodes``, ``blas_nodes``,
    ``normals``, ``normal_indices``, ``uvs``, ``uv_indices``, ``transforms``,
    ``materials``, ``textures``) and ``blob()`` returns an orn_scene_blob
    pointing at them."""

    def __init__(self, scene: Scene, row_major_transforms: bool = True, seed: int = 1244,
                 builder: str = "reference"):
        """builder: "reference" (bvh.zig's rules, the parity tree), "sah"
        (binned surface-area heuristic on the CPU) or "lbvh" (linear BVHs
        built on the GPU); the last two give fewer node visits and are not
        bit-exact with the reference's images."""
        lib = _lib.load()
        if builder not in ("reference", "sah", "lbvh"):
            raise ValueError("builder must be 'reference', 'sah' or 'lbvh'")
        mats = {id(m): i for i, m in enumerate(scene.materials)}
        texs = {id(t): i for i, t in enumerate(scene.textures)}
        keep = []

        def mat_index(m: Material) -> int:
            if id(m) not in mats:
                raise ValueError("material does not belong to the scene")
            return mats[id(m)]

        mdesc = (_lib.MaterialDesc * max(1, len(scene.materials)))()
        for i, m in enumerate(scene.materials):
            d = mdesc[i]
            if isinstance(m.albedo, Texture):
                d.albedo[:] = [1.0, 0.0, 1.0]
                d.texture = texs[id(m.albedo)]
            else:
                d.albedo[:] = [float(x) for x in list(m.albedo)[:3]]
                d.texture = _lib.NO_TEXTURE
            d.fuzz, d.ior, d.type = float(m.fuzz), float(m.ior), int(m.type)
        tdesc = (_lib.Texture * max(1, len(scene.textures)))()
        for i, t in enumerate(scene.textures):
            data = np.ascontiguousarray(t.data)
            keep.append(data)
            tdesc[i].data = data.ctypes.data
            tdesc[i].width, tdesc[i].height = t.width, t.height
            tdesc[i].bytes_per_row = t.bytes_per_row
            tdesc[i].format = _lib.TEXEL_RGBA8 if t.bytes_per_component == 1 else _lib.TEXEL_RGBA16F

        def fill_common(d, transform, aabb, material):
            d.transform[:] = [float(x) for x in np.asarray(transform, dtype=F32).reshape(16)]
            d.aabb_min[:] = [float(x) for x in aabb.min[:3]]
            d.aabb_max[:] = [float(x) for x in aabb.max[:3]]
            d.material = mat_index(material)

        sdesc = (_lib.SphereDesc * max(1, len(scene.spheres)))()
        for i, s in enumerate(scene.spheres):
            fill_common(sdesc[i], s.transform, s.aabb, s.material)
        mesh_index = {id(m): i for i, m in enumerate(scene.meshes)}
        medesc = (_lib.MeshDesc * max(1, len(scene.meshes)))()
        for i, m in enumerate(scene.meshes):
            d = medesc[i]
            arrays = [np.ascontiguousarray(a) for a in (m.vertices, m.vertex_indices, m.normals,
                                                          m.normal_indices, m.uvs, m.uv_indices)]
            keep.extend(arrays)
            d.vertices, d.vertices_len = _ptr(arrays[0]), len(arrays[0])
            d.vertex_indices, d.vertex_indices_len = _ptr(arrays[1]), len(arrays[1])
            d.normals, d.normals_len = _ptr(arrays[2]), len(arrays[2])
            d.normal_indices, d.normal_indices_len = _ptr(arrays[3]), len(arrays[3])
            d.uvs, d.uvs_len = _ptr(arrays[4]), len(arrays[4])
            d.uv_indices, d.uv_indices_len = _ptr(arrays[5]), len(arrays[5])
            fill_common(d, m.transform, m.aabb, m.material)
        idesc = (_lib.MeshInstanceDesc * max(1, len(scene.mesh_instances)))()
        for i, mi in enumerate(scene.mesh_instances):
            idesc[i].mesh = mesh_index[id(mi.mesh)]
            fill_common(idesc[i], mi.transform, mi.aabb, mi.material)
        desc = _lib.SceneDesc(C.cast(sdesc, C.c_void_p), len(scene.spheres),
                              C.cast(medesc, C.c_void_p), len(scene.meshes),
                              C.cast(idesc, C.c_void_p), len(scene.mesh_instances),
                              C.cast(mdesc, C.c_void_p), len(scene.materials),
                              C.cast(tdesc, C.c_void_p), len(scene.textures),
                              seed, 1 if row_major_transforms else 0,
                              {"reference": _lib.BVH_REFERENCE, "sah": _lib.BVH_SAH,
                               "lbvh": _lib.BVH_LBVH}[builder])
        handle = C.c_void_p()
        _lib.check(lib.orn_bvh_build(C.byref(desc), C.byref(handle)))
        try:
            blob = _lib.SceneBlob()
            _lib.check(lib.orn_bvh_get_blob(handle, C.byref(blob)))

            def arr(ptr, n, dtype, shape):
                if n == 0:
                    return np.zeros((0,) + shape, dtype=dtype)
                nbytes = n * np.dtype(dtype).itemsize * int(np.prod(shape) if shape else 1)
                raw = C.string_at(ptr, nbytes)
                return np.frombuffer(raw, dtype=dtype).reshape((n,) + shape).copy()

            self.tlas_nodes = arr(blob.tlas_nodes, blob.tlas_nodes_len, NODE_DTYPE, ())
            self.blas_nodes = arr(blob.blas_nodes, blob.blas_nodes_len, NODE_DTYPE, ())
            self.normals = arr(blob.normals, blob.normals_len, F32, (4,))
            self.normal_indices = arr(blob.normal_indices, blob.normal_indices_len, np.uint32, ())
            self.uvs = arr(blob.uvs, blob.uvs_len, F32, (2,))
            self.uv_indices = arr(blob.uv_indices, blob.uv_indices_len, np.uint32, ())
            self.transforms = arr(blob.transforms, blob.transforms_len, F32, (16,))
            self.materials = arr(blob.materials, blob.materials_len, MATERIAL_DTYPE, ())
            tex_ptrs = (_lib.Texture * max(1, blob.textures_len)).from_address(blob.textures) \
                if blob.textures_len else []
            by_ptr = {tdesc[i].data: scene.textures[i] for i in range(len(scene.textures))}
            self.textures = [by_ptr[tex_ptrs[i].data] for i in range(blob.textures_len)]
            self.scene_textures_count = blob.scene_textures_count
        finally:
            lib.orn_bvh_free(handle)
        self.row_major_transforms = row_major_transforms

    @classmethod
    def from_arrays(cls, **arrays) -> "Bvh":
        """A Bvh from flat arrays produced elsewhere (e.g. a fixture)."""
        self = cls.__new__(cls)
        for k, v in arrays.items():
            setattr(self, k, v)
        self.row_major_transforms = True
        return self

    def blob(self):
        """(orn_scene_blob, keep-alive list)."""
        keep = []

        def c(a, dtype):
            a = np.ascontiguousarray(a, dtype=dtype)
            keep.append(a)
            return _ptr(a), len(a)

        tex = (_lib.Texture * max(1, len(self.textures)))()
        for i, t in enumerate(self.textures):
            data = np.ascontiguousarray(t.data)
            keep.append(data)
            tex[i].data = data.ctypes.data
            tex[i].width, tex[i].height, tex[i].bytes_per_row = t.width, t.height, t.bytes_per_row
            tex[i].format = _lib.TEXEL_RGBA8 if t.bytes_per_component == 1 else _lib.TEXEL_RGBA16F
        keep.append(tex)
        b = _lib.SceneBlob()
        b.tlas_nodes, b.tlas_nodes_len = c(self.tlas_nodes, NODE_DTYPE)
        b.blas_nodes, b.blas_nodes_len = c(self.blas_nodes, NODE_DTYPE)
        b.normals, b.normals_len = c(self.normals, F32)
        b.normal_indices, b.normal_indices_len = c(self.normal_indices, np.uint32)
        b.uvs, b.uvs_len = c(self.uvs, F32)
        b.uv_indices, b.uv_indices_len = c(self.uv_indices, np.uint32)
        b.transforms, b.transforms_len = c(self.transforms, F32)
        b.materials, b.materials_len = c(self.materials, MATERIAL_DTYPE)
        b.textures = C.cast(tex, C.c_void_p).value if self.textures else None
        b.textures_len = len(self.textures)
        b.scene_textures_count = self.scene_textures_count
        return b, keep


# ---------------------------------------------------------------- path tracer


class Renderer:
    """The C-ABI context (orn_context) over a Bvh: a thin, explicit layer
    used by PathTracer, the tests and the benchmark."""

    def __init__(self, bvh: "Bvh", device: int = -1):
        self._lib = _lib.load()
        self.bvh = bvh
        blob, keep = bvh.blob()
        handle = C.c_void_p()
        _lib.check(self._lib.orn_create(C.byref(blob), device, C.byref(handle)))
        del keep
        self._ctx = handle
        self.width = self.height = 500

    def close(self):
        if getattr(self, "_ctx", None):
            self._lib.orn_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._ctx

    def _check(self, st):
        _lib.check(st, self._ctx)

    def set_state(self, state: "_lib.State"):
        self._check(self._lib.orn_set_state(self._ctx, C.byref(state)))

    def get_state(self) -> "_lib.State":
        s = _lib.State()
        self._check(self._lib.orn_get_state(self._ctx, C.byref(s)))
        return s

    def set_camera(self, camera: "_lib.Camera"):
        self._check(self._lib.orn_set_camera(self._ctx, C.byref(camera)))

    def set_resolution(self, width: int, height: int):
        self._check(self._lib.orn_set_resolution(self._ctx, width, height))
        self.width, self.height = width, height

    def render(self):
        self._check(self._lib.orn_render(self._ctx))

    def synchronize(self):
        self._check(self._lib.orn_synchronize(self._ctx))

    def framebuffer(self, dst: Optional[np.ndarray] = None) -> np.ndarray:
        n = self.width * self.height
        if dst is None:
            dst = np.empty((n, 4), dtype=F32)
        self._check(self._lib.orn_get_framebuffer(self._ctx, dst.ctypes.data, dst.size // 4))
        return dst

    def accumulation(self) -> np.ndarray:
        n = self.width * self.height
        dst = np.empty((n, 4), dtype=F32)
        self._check(self._lib.orn_get_accumulation(self._ctx, dst.ctypes.data, n))
        return dst

    def progress(self):
        n = self.width * self.height
        acc = np.empty((n, 4), dtype=F32)
        rng = np.empty(n, dtype=np.uint32)
        ci = C.c_float()
        self._check(self._lib.orn_get_progress(self._ctx, acc.ctypes.data, rng.ctypes.data, n, C.byref(ci)))
        return acc, rng, ci.value

    def set_progress(self, acc, rng, current_iteration):
        acc = np.ascontiguousarray(acc, dtype=F32)
        rng = np.ascontiguousarray(rng, dtype=np.uint32)
        self._check(self._lib.orn_set_progress(self._ctx, acc.ctypes.data, rng.ctypes.data, len(rng),
                                               float(current_iteration)))

    def peek_constant_params(self) -> "_lib.ConstantParams":
        cp = _lib.ConstantParams()
        self._check(self._lib.orn_peek_constant_params(self._ctx, C.byref(cp)))
        return cp

    def trace_rays(self, rays: np.ndarray, with_visits: bool = True):
        """rays: (n, 6) float32 origin+direction.  Returns (hits, visits)."""
        rays = np.ascontiguousarray(rays, dtype=F32).reshape(-1, 6)
        n = len(rays)
        hits = np.zeros(n, dtype=HIT_DTYPE)
        visits = np.zeros(n, dtype=np.uint32) if with_visits else None
        self._check(self._lib.orn_trace_rays(self._ctx, _ptr(rays), n, _ptr(hits),
                                             _ptr(visits) if with_visits else None))
        return hits, visits

    def enable_counters(self, enable: bool = True):
        self._check(self._lib.orn_enable_counters(self._ctx, 1 if enable else 0))

    def counters(self) -> dict:
        out = (C.c_uint64 * _lib.COUNTER_COUNT)()
        self._check(self._lib.orn_get_counters(self._ctx, out, _lib.COUNTER_COUNT))
        return dict(zip(_lib.COUNTER_NAMES, [int(x) for x in out]))

    def render_f64(self, spp: int) -> np.ndarray:
        """Per-pixel FP64 mean RGBA of `spp` passes from a fresh start
        (orn_render_f64)."""
        n = self.width * self.height
        out = np.empty((n, 4), dtype=np.float64)
        self._check(self._lib.orn_render_f64(self._ctx, spp, out.ctypes.data, n))
        return out

    def relmse(self, reference: np.ndarray, return_skipped: bool = False):
        """relMSE of the current accumulation against an FP64 mean image
        (non-finite pixels left out; with return_skipped, also their count)."""
        ref = np.ascontiguousarray(reference, dtype=np.float64).reshape(-1, 4)
        v = C.c_double()
        k = C.c_uint64()
        self._check(self._lib.orn_relmse(self._ctx, ref.ctypes.data, len(ref), C.byref(v), C.byref(k)))
        return (v.value, k.value) if return_skipped else v.value

    def stream(self) -> int:
        p = C.c_void_p()
        self._check(self._lib.orn_get_stream(self._ctx, C.byref(p)))
        return p.value or 0

    def launch_count(self) -> int:
        n = C.c_uint64()
        self._check(self._lib.orn_launch_count(self._ctx, C.byref(n)))
        return n.value

    def last_render_ms(self) -> float:
        ms = C.c_float()
        self._check(self._lib.orn_last_render_ms(self._ctx, C.byref(ms)))
        return ms.value

    def attach_cache(self, cache: Optional["RadianceCache"]):
        """Attach a RadianceCache for KERNEL_CACHED renders (None detaches)."""
        self._check(self._lib.orn_attach_cache(self._ctx, cache.handle if cache is not None else None))
        self._cache = cache   # keep it alive while attached

    @staticmethod
    def _wave_dict(c) -> dict:
        return {"shape": c.shape, "fetch": c.fetch, "steps": c.steps, "tuned": bool(c.tuned)}

    def wave_config(self) -> dict:
        """Launch parameters of KERNEL_WAVEFRONT renders (orn_wave_get_config)."""
        c = _lib.WaveConfig()
        self._check(self._lib.orn_wave_get_config(self._ctx, C.byref(c)))
        return self._wave_dict(c)

    def set_wave_config(self, shape: int = 0, fetch: int = 4, steps: int = 32):
        self._check(self._lib.orn_wave_set_config(self._ctx, C.byref(_lib.WaveConfig(shape, fetch, steps, 0))))

    def wave_tune(self, cache_path: Optional[str] = None) -> dict:
        """Autotune the wavefront's launch parameters for the current scene,
        camera, resolution and state (orn_wave_tune); returns the choice."""
        c = _lib.WaveConfig()
        path = str(cache_path).encode() if cache_path else None
        self._check(self._lib.orn_wave_tune(self._ctx, path, C.byref(c)))
        return self._wave_dict(c)


class RadianceCache:
    """The learned radiance cache (orn_cache_*): a 10-input, 5 x 64 ReLU,
    3-output MLP with frequency encoding, trained on the tensor cores.
    Parameters are FP32, six row-major [outputs][inputs] matrices in order
    (the output layer padded to 16 rows)."""

    PARAM_COUNT = _lib.CACHE_PARAM_COUNT

    def __init__(self, seed: int = 1, device: int = -1, **config):
        self._lib = _lib.load()
        cfg = _lib.CacheConfig()
        self._lib.orn_cache_default_config(C.byref(cfg))
        for k, v in config.items():
            setattr(cfg, k, v)
        h = C.c_void_p()
        st = self._lib.orn_cache_create(device, seed, C.byref(cfg), C.byref(h))
        if st != _lib.ORN_OK:
            raise _lib.OrnamentError(st, self._lib.orn_status_string(st).decode())
        self._h = h

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None):
            self._lib.orn_cache_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st):
        if st != _lib.ORN_OK:
            msg = self._lib.orn_cache_last_error(self._h).decode() or self._lib.orn_status_string(st).decode()
            raise _lib.OrnamentError(st, msg)

    def set_config(self, **config):
        cfg = _lib.CacheConfig()
        self._lib.orn_cache_default_config(C.byref(cfg))
        for k, v in config.items():
            setattr(cfg, k, v)
        self._check(self._lib.orn_cache_set_config(self._h, C.byref(cfg)))

    def params(self) -> np.ndarray:
        out = np.empty(self.PARAM_COUNT, dtype=F32)
        self._check(self._lib.orn_cache_get_params(self._h, out.ctypes.data, out.size))
        return out

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, dtype=F32).ravel()
        self._check(self._lib.orn_cache_set_params(self._h, p.ctypes.data, p.size))

    def infer(self, inputs: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(inputs, dtype=F32).reshape(-1, _lib.CACHE_INPUTS)
        out = np.empty((len(x), _lib.CACHE_OUTPUTS), dtype=F32)
        self._check(self._lib.orn_cache_infer(self._h, x.ctypes.data, len(x), out.ctypes.data))
        return out

    def gradients(self, inputs: np.ndarray, targets: np.ndarray):
        """(grads, summed loss) of the summed relative-L2 loss; no update."""
        x = np.ascontiguousarray(inputs, dtype=F32).reshape(-1, _lib.CACHE_INPUTS)
        t = np.ascontiguousarray(targets, dtype=F32).reshape(-1, _lib.CACHE_OUTPUTS)
        g = np.empty(self.PARAM_COUNT, dtype=F32)
        loss = C.c_float()
        self._check(self._lib.orn_cache_gradients(self._h, x.ctypes.data, t.ctypes.data, len(x), g.ctypes.data,
                                                  C.byref(loss)))
        return g, loss.value

    def train(self, inputs: np.ndarray, targets: np.ndarray) -> float:
        """One Adam step on the mean loss; returns the summed loss."""
        x = np.ascontiguousarray(inputs, dtype=F32).reshape(-1, _lib.CACHE_INPUTS)
        t = np.ascontiguousarray(targets, dtype=F32).reshape(-1, _lib.CACHE_OUTPUTS)
        loss = C.c_float()
        self._check(self._lib.orn_cache_train(self._h, x.ctypes.data, t.ctypes.data, len(x), C.byref(loss)))
        return loss.value

    def stats(self):
        steps, frames, loss = C.c_uint64(), C.c_uint64(), C.c_float()
        self._check(self._lib.orn_cache_stats(self._h, C.byref(steps), C.byref(frames), C.byref(loss)))
        return {"steps": steps.value, "frames": frames.value, "last_loss": loss.value}


class Batch:
    """Renders one render() of many Renderers (up to 64, one device, same
    semantics) in a single persistent launch replayed as a CUDA graph
    (orn_batch_*).  Each renderer's image and progress end as its own
    render() would leave them."""

    def __init__(self, renderers):
        self._lib = _lib.load()
        self.renderers = list(renderers)
        arr = (C.c_void_p * len(self.renderers))(*[r.handle.value for r in self.renderers])
        h = C.c_void_p()
        st = self._lib.orn_batch_create(arr, len(self.renderers), C.byref(h))
        if st != _lib.ORN_OK:
            raise _lib.OrnamentError(st, self._lib.orn_status_string(st).decode())
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._lib.orn_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st):
        if st != _lib.ORN_OK:
            msg = self._lib.orn_batch_last_error(self._h).decode() or self._lib.orn_status_string(st).decode()
            raise _lib.OrnamentError(st, msg)

    def render(self):
        self._check(self._lib.orn_batch_render(self._h))

    def synchronize(self):
        self._check(self._lib.orn_batch_synchronize(self._h))

    def last_render_ms(self) -> float:
        ms = C.c_float()
        self._check(self._lib.orn_batch_last_render_ms(self._h, C.byref(ms)))
        return ms.value

    def config(self) -> dict:
        c = _lib.BatchConfig()
        self._check(self._lib.orn_batch_get_config(self._h, C.byref(c)))
        return {"block": c.block, "blocks_per_sm": c.blocks_per_sm, "shade_threshold": c.shade_threshold,
                "tuned": bool(c.tuned)}

    def set_config(self, block=128, blocks_per_sm=6, shade_threshold=8):
        c = _lib.BatchConfig(block, blocks_per_sm, shade_threshold, 0)
        self._check(self._lib.orn_batch_set_config(self._h, C.byref(c)))

    def tune(self, cache_path: Optional[str] = None) -> dict:
        c = _lib.BatchConfig()
        path = str(cache_path).encode() if cache_path else None
        self._check(self._lib.orn_batch_tune(self._h, path, C.byref(c)))
        return {"block": c.block, "blocks_per_sm": c.blocks_per_sm, "shade_threshold": c.shade_threshold,
                "tuned": bool(c.tuned)}


class PathTracer:
    """The CUDA backend behind the PathTracer surface
    (src/hip_backend/path_tracer.zig:12-236).

    ``scene`` and ``state`` are public like in the reference: change
    ``state`` through its setters and ``scene.camera`` through
    setLookAt/setAspectRatio; render() picks the changes up."""

    def __init__(self, scene: Scene, device: int = -1, bvh: Optional[Bvh] = None):
        self.scene = scene
        self.state = State()
        self.bvh = bvh if bvh is not None else Bvh(scene, row_major_transforms=True)
        self.renderer = Renderer(self.bvh, device)
        self._applied_resolution = None

    # -- reference surface
    def deinit(self):
        self.renderer.close()

    def setResolution(self, resolution: Resolution):
        self.state.setResolution(resolution)
        self.renderer.set_resolution(resolution.width, resolution.height)
        self._applied_resolution = (resolution.width, resolution.height)

    def _sync_state(self):
        r = self.state.resolution
        if self._applied_resolution != (r.width, r.height):
            self.setResolution(r)
        self.renderer.set_state(self.state.to_struct())
        if self.scene.camera.dirty:
            self.renderer.set_camera(self.scene.camera.to_struct())
            self.scene.camera.dirty = False

    def render(self):
        self._sync_state()
        self.renderer.render()

    def getFrameBuffer(self, dst: Optional[np.ndarray] = None) -> np.ndarray:
        r = self.state.resolution
        if dst is not None and (dst.dtype != F32 or not dst.flags.c_contiguous or dst.size < 4 * r.pixel_count()):
            raise ValueError("dst must be a contiguous float32 array of pixel_count x 4")
        self._sync_state()
        return self.renderer.framebuffer(dst)

    # -- extensions
    def getProgress(self):
        self._sync_state()
        return self.renderer.progress()

    def setProgress(self, acc, rng, current_iteration):
        self._sync_state()
        self.renderer.set_progress(acc, rng, current_iteration)

    def traceRays(self, rays: np.ndarray, with_visits: bool = True):
        self._sync_state()
        return self.renderer.trace_rays(rays, with_visits)


HIT_DTYPE = np.dtype([("hit", np.uint32), ("t", F32), ("material_index", np.uint32), ("node_type", np.uint32),
                      ("inverted_transform_id", np.uint32), ("tri_id", np.uint32), ("uv", F32, 2)])
assert HIT_DTYPE.itemsize == 32
