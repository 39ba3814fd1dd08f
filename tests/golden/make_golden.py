"""Generates tests/golden/golden_v1.npz from the reference itself.

Run where the zig_ornament sources are available (the directory
oracle/build_oracle.py looks in; ORN_REFERENCE_DIR overrides it):

    python tests/golden/make_golden.py

It compiles the reference's HIP kernel source unmodified for the host
(oracle/build_oracle.py, through oracle/shim) and records:
  * unit vectors: RndGen draws (random.hip.h:8-30), safe_invdir edge cases
    (bvh.hip.h:43-52), aabb_hit / triangle_hit / sphere_hit cases
    (bvh.hip.h:54-143);
  * a small scene's flat arrays (built by this project's orn_bvh_build, the
    shared input) and the reference's outputs on it: Bvh::hit on 4096 rays,
    and PathTracer.render-style passes (accumulation, RNG states,
    framebuffer) for several State settings, with glibc transcendentals and
    with the project's portable ones.
The fixture lets the tests pin the oracle and the GPU kernels without the
reference sources present.
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import oracle_lib as ol  # noqa: E402
from zig_ornament_gb300 import scenes, ornament  # noqa: E402

OUT = Path(__file__).resolve().parent / "golden_v1.npz"
W, H = 96, 64


def ptr(a):
    return a.ctypes.data


def unit_cases(ref, rs):
    lib = ref.lib
    for fn in ("ref_pcg", "ref_safe_invdir", "ref_triangle_hit", "ref_sphere_hit", "ref_aabb_hit"):
        getattr(lib, fn).restype = C.c_int
    lib.ref_pcg.argtypes = [C.c_uint32, C.c_size_t, C.c_void_p, C.c_void_p]
    for fn in ("ref_safe_invdir", "ref_triangle_hit", "ref_sphere_hit", "ref_aabb_hit"):
        getattr(lib, fn).argtypes = [C.c_void_p, C.c_size_t, C.c_void_p]
    out = {}
    seeds = np.array([0, 1, 2, 255, 12345, 2073599, 0x7fffffff, 0xffffffff], np.uint32)
    u = np.zeros((len(seeds), 64), np.uint32)
    f = np.zeros((len(seeds), 64), np.float32)
    for i, s in enumerate(seeds):
        uu = np.zeros(64, np.uint32)
        ff = np.zeros(64, np.float32)
        lib.ref_pcg(int(s), 64, ptr(uu), ptr(ff))
        u[i], f[i] = uu, ff
    out.update(pcg_seeds=seeds, pcg_u32=u, pcg_f32=f)
    specials = [0.0, -0.0, 1e-5, -1e-5, 1.0000001e-5, -1.0000001e-5, 9.99e-6, -9.99e-6, 1e-30, -1e-30,
                1.0, -1.0, 0.5, -123.25, 3e38, -3e38]
    d = np.array([[a, b, c] for a in specials for b in specials[:4] for c in specials[:3]], np.float32)
    d = np.concatenate([d, rs.normal(size=(64, 3)).astype(np.float32)])
    inv = np.zeros_like(d)
    lib.ref_safe_invdir(ptr(d), len(d), ptr(inv))
    out.update(invdir_in=d, invdir_out=inv)
    # triangle cases: random rays against random triangles, plus edges/vertices
    n = 512
    tri = np.zeros((n, 17), np.float32)
    tri[:, 0:3] = rs.normal(size=(n, 3)) * 3
    v = rs.normal(size=(n, 9)).astype(np.float32)
    target = (v[:, 0:3] + v[:, 3:6] + v[:, 6:9]) / 3 + rs.normal(size=(n, 3)) * 0.5
    tri[:, 3:6] = target - tri[:, 0:3]
    tri[:, 6:15] = v
    tri[:, 15] = 0.001
    tri[:, 16] = 3.40282e38
    # exact edge / vertex hits and a parallel ray
    tri[:8, 6:15] = [0, 0, 0, 1, 0, 0, 0, 1, 0]
    tri[:8, 0:3] = [[0, 0, 1], [1, 0, 1], [0, 1, 1], [0.5, 0.5, 1], [0.25, 0.25, 1], [2, 2, 1], [0, 0, 1], [0.3, 0.3, 0]]
    tri[:8, 3:6] = [[0, 0, -1]] * 6 + [[1, 0, 0], [1, 0, 0]]
    tri[8:16, 16] = rs.uniform(0.5, 3.0, 8)
    tout = np.zeros((n, 3), np.float32)
    lib.ref_triangle_hit(ptr(tri), n, ptr(tout))
    out.update(tri_in=tri, tri_out=tout)
    sph = np.zeros((n, 8), np.float32)
    sph[:, 0:3] = rs.normal(size=(n, 3)) * 3
    sph[:, 3:6] = -sph[:, 0:3] + rs.normal(size=(n, 3)) * 0.8
    sph[:, 6] = 0.001
    sph[:, 7] = 3.40282e38
    sph[:16, 0:3] = rs.normal(size=(16, 3)) * 0.3   # origins inside the sphere
    sph[16:24, 7] = rs.uniform(0.5, 4.0, 8)
    sout = np.zeros(n, np.float32)
    lib.ref_sphere_hit(ptr(sph), n, ptr(sout))
    out.update(sphere_in=sph, sphere_out=sout)
    box = np.zeros((n, 14), np.float32)
    lo = rs.normal(size=(n, 3)).astype(np.float32)
    box[:, 0:3] = lo
    box[:, 3:6] = lo + rs.uniform(0, 2, (n, 3))
    dirs = rs.normal(size=(n, 3)).astype(np.float32)
    dirs[:32, rs.integers(0, 3, 32)] = 0.0
    orig = rs.normal(size=(n, 3)).astype(np.float32) * 3
    invd = np.zeros_like(dirs)
    lib.ref_safe_invdir(ptr(dirs), n, ptr(invd))
    box[:, 6:9] = invd
    box[:, 9:12] = (-orig) * invd
    box[:, 12] = 0.001
    box[:, 13] = 3.40282e38
    box[32:64, 13] = rs.uniform(0.1, 5, 32)
    bout = np.zeros((n, 2), np.float32)
    lib.ref_aabb_hit(ptr(box), n, ptr(bout))
    out.update(aabb_in=box, aabb_out=bout)
    return out


def random_rays(scene, rs, n):
    cam = scene.camera
    o = np.asarray(cam.origin[:3], np.float32)
    target = rs.uniform(-4, 4, (n, 3)).astype(np.float32)
    target[:, 1] = rs.uniform(-0.5, 4.5, n)
    origins = o + rs.normal(size=(n, 3)).astype(np.float32) * 0.5
    origins[: n // 4] = rs.uniform(-3, 3, (n // 4, 3))   # some rays start inside the scene
    d = target - origins
    d[: n // 16] = rs.normal(size=(n // 16, 3))
    return np.concatenate([origins, d], axis=1).astype(np.float32)


def main():
    if not ol.reference_available():
        raise SystemExit("zig_ornament sources not found: set ORN_REFERENCE_DIR")
    rs = np.random.default_rng(20261203)
    ref = ol.Reference(portable_math=False)
    refp = ol.Reference(portable_math=True)
    out = unit_cases(ref, rs)
    scene = scenes.small_test_scene(W, H)
    bvh = ornament.Bvh(scene)
    for k in ("tlas_nodes", "blas_nodes", "normals", "normal_indices", "uvs", "uv_indices", "transforms",
              "materials"):
        out["scene_" + k] = getattr(bvh, k)
    tex_src = {id(t): i for i, t in enumerate(scene.textures)}
    out["scene_texture_map"] = np.array([tex_src[id(t)] for t in bvh.textures], np.int32)
    for i, t in enumerate(scene.textures):
        out[f"scene_texture_{i}"] = t.data
    out["scene_textures_count"] = np.array(bvh.scene_textures_count, np.uint32)
    out["scene_counts"] = np.array([len(scene.spheres), len(scene.meshes), len(scene.mesh_instances),
                                    sum(len(m.vertex_indices) // 3 for m in scene.meshes)], np.int64)
    cam = scene.camera.to_struct()
    out["camera"] = np.frombuffer(bytes(cam), np.uint8).copy()
    rays = random_rays(scene, rs, 4096)
    out["rays"] = rays
    hits = ref.trace_rays(bvh, rays)
    out["ray_hits"] = hits
    # render cases: (name, spp, ci_start, depth, gamma, flip, from_case)
    cases = [("fused1", 1, 1.0, 8, 1.0, False, None), ("pass5", 5, 1.0, 8, 2.2, False, None),
             ("cont3", 3, 6.0, 8, 2.2, False, "pass5"), ("flip4", 4, 1.0, 10, 2.2, True, None)]
    for math_name, r in (("libm", ref), ("pmath", refp)):
        states = {}
        for name, spp, ci, depth, gamma, flip, base in cases:
            cp = ol.make_params(scene.camera, W, H, depth=depth, flip_y=flip, gamma=gamma,
                                textures_count=bvh.scene_textures_count)
            acc0, rng0 = (states[base][0], states[base][1]) if base else (None, None)
            acc, rng, fb = r.render(bvh, cp, spp, ci_start=ci, acc=acc0, rng=rng0)
            states[name] = (acc, rng, fb)
            out[f"render_{math_name}_{name}_acc"] = acc
            out[f"render_{math_name}_{name}_rng"] = rng
            out[f"render_{math_name}_{name}_fb"] = fb
    out["render_cases"] = np.array([f"{n}|{s}|{c}|{d}|{g}|{int(f)}|{b or ''}" for n, s, c, d, g, f, b in cases])
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT} ({OUT.stat().st_size / 1e3:.0f} kB)")


if __name__ == "__main__":
    main()
