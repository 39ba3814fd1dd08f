"""Seeded synthetic scenes for the benchmark configurations and the tests.

No dataset is involved: every mesh, texture, transform and material is
generated from a numpy PCG64 stream with a fixed seed.

  spheres_scene          the "Ray Tracing in One Weekend" sphere field
                         (glfw_example/examples.zig:33-91 shape; by default a
                         22x22 grid a,b in [-11, 11) without the exclusion
                         zone, ``reference_grid=True`` gives the example's
                         21x21 grid that skips centres near (4, 0.2, 0)).
  instanced_meshes_scene 8 BLAS (subdivided icospheres and tori of radius 4,
                         10k-80k triangles, per-vertex normals and UVs), 256 instances
                         with random scale 0.5-3, random rotation and a
                         translation in a 100^3 box, sphere-field materials,
                         4 procedural 1024^2 RGBA8 textures, one emissive
                         quad of radiance 15.
  small_test_scene       a few spheres, meshes, instances and small textures
                         (parity tests).
  large_scene            4096 instances over 32 BLAS (~10M triangles), 8 quads.
  batch_scenes           64 scenes of uneven size for the batched renderer.
  cornell_box_scene      a closed room lit by one ceiling light (radiance cache).
"""
from __future__ import annotations

import math

import numpy as np

from . import _lib
from .ornament import (F32, Scene, Camera, f32x4, mul, scaling, translation, matFromQuat, getSphereTexCoord)

# ------------------------------------------------------------------ geometry


def icosphere(freq: int):
    """Geodesic sphere: each icosahedron face split into freq^2 triangles,
    vertices projected on the unit sphere.  Returns (vertices(n,4), normals(n,4),
    uvs(n,2), indices)."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    base = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t],
                     [0, 1, -t], [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], dtype=np.float64)
    faces = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4],
                      [11, 10, 2], [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8],
                      [3, 8, 9], [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]])
    n = freq
    # barycentric lattice of one face
    ij = [(i, j) for i in range(n + 1) for j in range(n + 1 - i)]
    lid = {p: k for k, p in enumerate(ij)}
    tris = []
    for i in range(n):
        for j in range(n - i):
            tris.append((lid[(i, j)], lid[(i + 1, j)], lid[(i, j + 1)]))
            if j < n - i - 1:
                tris.append((lid[(i + 1, j)], lid[(i + 1, j + 1)], lid[(i, j + 1)]))
    tris = np.array(tris, dtype=np.int64)
    w = np.array([(n - i - j, i, j) for i, j in ij], dtype=np.float64) / n
    verts, idx = [], []
    for f, face in enumerate(faces):
        p = w @ base[face]
        p /= np.linalg.norm(p, axis=1, keepdims=True)
        idx.append(tris + f * len(ij))
        verts.append(p)
    p = np.concatenate(verts).astype(F32)
    idx = np.concatenate(idx).reshape(-1).astype(np.uint32)
    v4 = np.concatenate([p, np.ones((len(p), 1), F32)], axis=1)
    n4 = np.concatenate([p, np.zeros((len(p), 1), F32)], axis=1)
    theta = np.arccos(np.clip(-p[:, 1].astype(np.float64), -1, 1))
    phi = np.arctan2(-p[:, 2].astype(np.float64), p[:, 0].astype(np.float64)) + math.pi
    uv = np.stack([phi / (2 * math.pi), theta / math.pi], axis=1).astype(F32)
    return v4, n4, uv, idx


def torus(nu: int, nv: int, major: float = 1.0, minor: float = 0.35):
    """Torus around the y axis with nu x nv quads (2*nu*nv triangles)."""
    u = np.arange(nu) / nu * 2 * math.pi
    v = np.arange(nv) / nv * 2 * math.pi
    U, V = np.meshgrid(u, v, indexing="ij")
    cx, cz = np.cos(U), np.sin(U)
    px = (major + minor * np.cos(V)) * cx
    py = minor * np.sin(V)
    pz = (major + minor * np.cos(V)) * cz
    nx, ny, nz = np.cos(V) * cx, np.sin(V), np.cos(V) * cz
    p = np.stack([px, py, pz], -1).reshape(-1, 3).astype(F32)
    nrm = np.stack([nx, ny, nz], -1).reshape(-1, 3).astype(F32)
    uv = np.stack([U / (2 * math.pi), V / (2 * math.pi)], -1).reshape(-1, 2).astype(F32)
    i = np.arange(nu)[:, None]
    j = np.arange(nv)[None, :]
    a = (i * nv + j)
    b = (((i + 1) % nu) * nv + j)
    c = (((i + 1) % nu) * nv + (j + 1) % nv)
    d = (i * nv + (j + 1) % nv)
    idx = np.stack([a, b, c, a, c, d], -1).reshape(-1).astype(np.uint32)
    v4 = np.concatenate([p, np.ones((len(p), 1), F32)], 1)
    n4 = np.concatenate([nrm, np.zeros((len(p), 1), F32)], 1)
    return v4, n4, uv, idx


def random_rotation(rng: np.random.Generator) -> np.ndarray:
    """Uniformly distributed rotation (Shoemake's quaternion method)."""
    u1, u2, u3 = rng.random(3)
    q = (math.sqrt(1 - u1) * math.sin(2 * math.pi * u2), math.sqrt(1 - u1) * math.cos(2 * math.pi * u2),
         math.sqrt(u1) * math.sin(2 * math.pi * u3), math.sqrt(u1) * math.cos(2 * math.pi * u3))
    return matFromQuat(q)


# ------------------------------------------------------------------ textures


def checker_texture(size: int, rng: np.random.Generator, squares: int = 16) -> np.ndarray:
    c0 = (rng.random(3) * 255).astype(np.uint8)
    c1 = (rng.random(3) * 255).astype(np.uint8)
    y, x = np.mgrid[0:size, 0:size]
    m = ((x * squares // size) + (y * squares // size)) % 2
    img = np.where(m[..., None] == 0, c0, c1).astype(np.uint8)
    return np.concatenate([img, np.full((size, size, 1), 255, np.uint8)], axis=2)


def value_noise_texture(size: int, rng: np.random.Generator, octaves: int = 4) -> np.ndarray:
    acc = np.zeros((size, size), np.float64)
    amp, total = 1.0, 0.0
    for o in range(octaves):
        cells = 4 * (2 ** o)
        lattice = rng.random((cells + 1, cells + 1))
        t = np.linspace(0, cells, size, endpoint=False)
        i = t.astype(int)
        f = t - i
        f = f * f * (3 - 2 * f)
        a = lattice[i][:, i]
        b = lattice[i][:, i + 1]
        c = lattice[i + 1][:, i]
        d = lattice[i + 1][:, i + 1]
        fx, fy = f[None, :], f[:, None]
        acc += amp * ((a * (1 - fx) + b * fx) * (1 - fy) + (c * (1 - fx) + d * fx) * fy)
        total += amp
        amp *= 0.5
    acc /= total
    tint = 0.3 + 0.7 * rng.random(3)
    img = (acc[..., None] * tint[None, None, :] * 255).clip(0, 255).astype(np.uint8)
    return np.concatenate([img, np.full((size, size, 1), 255, np.uint8)], axis=2)


# ------------------------------------------------------------------ materials


def random_material(scene: Scene, rng: np.random.Generator, textures=(), textured_fraction=0.0,
                    mix=(0.8, 0.95), fuzz_max=0.5):
    """Sphere-field material mix: lambertian (albedo U^2 per channel), metal
    (albedo U(0.5, 1), fuzz U(0, fuzz_max)), dielectric (ior 1.5); `mix`
    holds the cumulative lambertian and metal fractions."""
    choose = rng.random()
    if choose < mix[0]:
        if textures and rng.random() < textured_fraction:
            return scene.lambertian(textures[int(rng.integers(len(textures)))])
        return scene.lambertian(tuple((rng.random(3) * rng.random(3)).tolist()) + (1.0,))
    if choose < mix[1]:
        return scene.metal(tuple((0.5 + 0.5 * rng.random(3)).tolist()) + (1.0,), float(fuzz_max * rng.random()))
    return scene.dielectric(1.5)


# ------------------------------------------------------------------ scenes


def spheres_scene(width=640, height=360, seed=0, reference_grid=False) -> Scene:
    scene = Scene()
    rng = np.random.default_rng(seed)
    scene.camera = Camera(f32x4(13, 2, 3, 1), f32x4(0, 0, 0, 1), f32x4(0, 1, 0, 0), width / height, 20.0, 0.1, 10.0)
    scene.attachSphere(scene.createSphere(f32x4(0, -1000, 0, 1), 1000.0, scene.lambertian((0.5, 0.5, 0.5, 1.0))))
    grid = range(-11, 10) if reference_grid else range(-11, 11)
    for a in grid:
        for b in grid:
            choose = rng.random()
            center = f32x4(a + 0.9 * rng.random(), 0.2, b + 0.9 * rng.random(), 1.0)
            if reference_grid and np.linalg.norm(center[:3] - np.array([4.0, 0.2, 0.0], F32)) <= 0.9:
                continue
            if choose < 0.8:
                mat = scene.lambertian(tuple((rng.random(3) * rng.random(3)).tolist()) + (1.0,))
            elif choose < 0.95:
                mat = scene.metal(tuple((0.5 + 0.5 * rng.random(3)).tolist()) + (1.0,), float(0.5 * rng.random()))
            else:
                mat = scene.dielectric(1.5)
            scene.attachSphere(scene.createSphere(center, 0.2, mat))
    scene.attachSphere(scene.createSphere(f32x4(0, 1, 0, 1), 1.0, scene.dielectric(1.5)))
    scene.attachSphere(scene.createSphere(f32x4(-4, 1, 0, 1), 1.0, scene.lambertian((0.4, 0.2, 0.1, 1.0))))
    scene.attachSphere(scene.createSphere(f32x4(4, 1, 0, 1), 1.0, scene.metal((0.7, 0.6, 0.5, 1.0), 0.0)))
    return scene


def _blas_mesh(rng, target_tris, radius):
    if rng.random() < 0.5:
        freq = max(1, int(round(math.sqrt(target_tris / 20.0))))
        v, n, uv, idx = icosphere(freq)
    else:
        nv = max(3, int(round(math.sqrt(target_tris / 4.0))))
        v, n, uv, idx = torus(2 * nv, nv)
    v = v.copy()
    v[:, :3] *= F32(radius)
    return v, n, uv, idx


def instanced_meshes_scene(width=1920, height=1080, seed=1, n_blas=8, n_instances=256,
                           tri_range=(10_000, 80_000), n_textures=4, texture_size=1024,
                           box=100.0, n_lights=1, textured_fraction=0.25, mix=(0.8, 0.95),
                           blas_radius=4.0, fuzz_max=0.5, light_size=40.0) -> Scene:
    scene = Scene()
    rng = np.random.default_rng(seed)
    textures = []
    for k in range(n_textures):
        img = checker_texture(texture_size, rng) if k % 2 == 0 else value_noise_texture(texture_size, rng)
        textures.append(scene.createTexture(img, texture_size, texture_size, 4, 1, False, 1.0))
    half = box / 2.0

    def random_transform():
        s = float(rng.uniform(0.5, 3.0))
        t = rng.uniform(-half, half, 3)
        return mul(mul(scaling(s, s, s), random_rotation(rng)), translation(*t))

    meshes = []
    lo, hi = math.log(tri_range[0]), math.log(tri_range[1])
    for _ in range(n_blas):
        target = math.exp(rng.uniform(lo, hi))
        v, n, uv, idx = _blas_mesh(rng, target, blas_radius)
        mat = random_material(scene, rng, textures, textured_fraction, mix, fuzz_max)
        m = scene.createMesh(v, idx, n, idx, uv, idx, random_transform(), mat)
        scene.attachMesh(m)
        meshes.append(m)
    for _ in range(n_instances):
        base = meshes[int(rng.integers(len(meshes)))]
        mat = random_material(scene, rng, textures, textured_fraction, mix, fuzz_max)
        scene.attachMeshInstance(scene.createMeshInstance(base, random_transform(), mat))
    light = scene.diffuseLight((15.0, 15.0, 15.0, 1.0))
    for k in range(n_lights):
        cx = 0.0 if n_lights == 1 else float(rng.uniform(-half * 0.6, half * 0.6))
        cz = 0.0 if n_lights == 1 else float(rng.uniform(-half * 0.6, half * 0.6))
        scene.attachMesh(scene.createPlaneMesh(f32x4(cx, half + 20.0, cz, 1), light_size, light_size,
                                               f32x4(0, -1, 0, 0), light))
    scene.camera = Camera(f32x4(0, 0.45 * box, 1.9 * box, 1), f32x4(0, 0, 0, 1), f32x4(0, 1, 0, 0),
                          width / height, 40.0, 0.0, 1.9 * box)
    return scene


def large_scene(width=3840, height=2160, seed=4, n_blas=32, n_instances=4096, total_tris=10_000_000,
                texture_size=1024) -> Scene:
    """The large configuration: `n_instances` instances over `n_blas`
    icosphere/torus BLAS totalling about `total_tris` triangles (each BLAS
    log-uniform within x0.7..x1.4 of the mean share), materials 40 %
    dielectric / 30 % metal (fuzz U(0, 0.3)) / 30 % textured lambertian,
    8 emissive quads.  The box grows to 250 so the instance density matches
    the 1080p scene's 256 instances in 100^3, and the quads grow with it."""
    per = total_tris / n_blas
    return instanced_meshes_scene(width, height, seed=seed, n_blas=n_blas, n_instances=n_instances - n_blas,
                                  tri_range=(0.7 * per, 1.4 * per), n_textures=4, texture_size=texture_size,
                                  box=250.0, n_lights=8, textured_fraction=1.0, mix=(0.3, 0.6), fuzz_max=0.3,
                                  light_size=100.0)


BATCH_RESOLUTIONS = ((256, 256), (640, 360), (1280, 720), (1920, 1080))


def batch_scenes(count=64, seed=2, tri_range=(1_000, 2_000_000), instance_range=(1, 1024), spp_range=(16, 256),
                 resolutions=BATCH_RESOLUTIONS, texture_size=256):
    """The batched-rendering workload: `count` independent instanced-mesh
    scenes (as instanced_meshes_scene), each with its total BLAS triangle
    count log-uniform in `tri_range` (spread over up to 8 BLAS), an instance
    count log-uniform in `instance_range`, a resolution drawn from
    `resolutions` and a sample count log-uniform in `spp_range`.  Returns a
    list of (scene, width, height, spp).  Textures are `texture_size`^2
    (procedural, as in the 1080p scene)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        tris = math.exp(rng.uniform(math.log(tri_range[0]), math.log(tri_range[1])))
        n_blas = int(min(8, max(1, tris // 2_000)))
        per = tris / n_blas
        inst = int(round(math.exp(rng.uniform(math.log(instance_range[0]), math.log(instance_range[1])))))
        w, h = resolutions[int(rng.integers(len(resolutions)))]
        spp = int(round(math.exp(rng.uniform(math.log(spp_range[0]), math.log(spp_range[1])))))
        scene = instanced_meshes_scene(w, h, seed=int(rng.integers(1 << 30)), n_blas=n_blas,
                                       n_instances=max(inst - n_blas, 0),
                                       tri_range=(max(per * 0.8, 80.0), per * 1.25), n_textures=2,
                                       texture_size=texture_size)
        out.append((scene, w, h, spp))
    return out


def cornell_box_scene(width=640, height=360, light_radiance=8.0, light_size=3.0) -> Scene:
    """A closed 10 x 10 x 10 room (white floor, ceiling and back/front walls,
    red left and green right walls) lit by one square ceiling light, with a
    glass, a brushed-metal and a white sphere; the camera is inside, so every
    path bounces until it reaches the light or the depth limit.  Used to
    measure the radiance cache where multi-bounce light dominates."""
    scene = Scene()
    white = scene.lambertian((0.73, 0.73, 0.73, 1.0))
    red = scene.lambertian((0.65, 0.05, 0.05, 1.0))
    green = scene.lambertian((0.12, 0.45, 0.15, 1.0))
    light = scene.diffuseLight((light_radiance, light_radiance, light_radiance, 1.0))
    walls = [((0, 0, 0), (0, 1, 0), white), ((0, 10, 0), (0, -1, 0), white), ((0, 5, -5), (0, 0, 1), white),
             ((0, 5, 5), (0, 0, -1), white), ((-5, 5, 0), (1, 0, 0), red), ((5, 5, 0), (-1, 0, 0), green)]
    for c, n, m in walls:
        scene.attachMesh(scene.createPlaneMesh(f32x4(*c, 1), 10.0, 10.0, f32x4(*n, 0), m))
    scene.attachMesh(scene.createPlaneMesh(f32x4(0, 9.98, 0, 1), light_size, light_size, f32x4(0, -1, 0, 0), light))
    scene.attachSphere(scene.createSphere(f32x4(-2.2, 1.5, -1.5, 1), 1.5, scene.dielectric(1.5)))
    scene.attachSphere(scene.createSphere(f32x4(2.2, 1.5, -0.5, 1), 1.5,
                                          scene.metal((0.8, 0.7, 0.6, 1.0), 0.3)))
    scene.attachSphere(scene.createSphere(f32x4(0.0, 1.0, 1.5, 1), 1.0, white))
    scene.camera = Camera(f32x4(0, 5, 4.9, 1), f32x4(0, 4, -5, 1), f32x4(0, 1, 0, 0), width / height, 75.0, 0.0, 10.0)
    return scene


def small_test_scene(width=96, height=64, seed=7, textured=True, with_spheres=True) -> Scene:
    """A scene that exercises every node type, material and texture path."""
    scene = Scene()
    rng = np.random.default_rng(seed)
    textures = []
    if textured:
        textures.append(scene.createTexture(checker_texture(32, rng, squares=4), 32, 32))
        img16 = (value_noise_texture(16, rng).astype(np.float32) / 255.0 * 2.0).astype(np.float16)
        textures.append(scene.createTexture(img16, 16, 16, 4, 2, True, 1.0))
    scene.camera = Camera(f32x4(0, 3, 14, 1), f32x4(0, 0.5, 0, 1), f32x4(0, 1, 0, 0), width / height, 35.0, 0.2, 12.0)
    if with_spheres:
        scene.createSphere(f32x4(0, -100.5, 0, 1), 100.0, scene.lambertian((0.6, 0.6, 0.5, 1.0)))
        for k in range(6):
            c = f32x4(-3 + 1.2 * k, 0.1, 1.5 * math.sin(k), 1)
            scene.createSphere(c, 0.45, random_material(scene, rng, textures, 0.5))
        if textures:
            scene.createSphere(f32x4(0, 2.5, -2, 1), 0.8, scene.lambertian(textures[1]))
    v, n, uv, idx = icosphere(4)
    ico = scene.createMesh(v, idx, n, idx, uv, idx, mul(scaling(0.7, 0.7, 0.7), translation(-2.0, 1.2, -1.0)),
                           scene.metal((0.8, 0.7, 0.6, 1.0), 0.1))
    v, n, uv, idx = torus(24, 12)
    tor = scene.createMesh(v, idx, n, idx, uv, idx, mul(scaling(0.8, 0.8, 0.8), translation(2.0, 1.0, -1.0)),
                           scene.lambertian(textures[0]) if textures else scene.lambertian((0.2, 0.7, 0.3, 1.0)))
    for k in range(5):
        t = mul(mul(scaling(0.5, 0.5, 0.5), random_rotation(rng)), translation(-2.5 + 1.25 * k, 2.0, 1.0))
        scene.createMeshInstance(ico if k % 2 == 0 else tor, t, random_material(scene, rng, textures, 0.5))
    scene.createMeshInstance(tor, mul(scaling(0.6, 0.6, 0.6), translation(0.0, 0.4, 2.5)), scene.dielectric(1.5))
    scene.createPlaneMesh(f32x4(0, 4.5, 0, 1), 3.0, 3.0, f32x4(0, -1, 0, 0), scene.diffuseLight((6.0, 6.0, 6.0, 1.0)))
    return scene
