"""The CPU oracle against the reference: committed golden vectors (always)
and the reference's own HIP kernels compiled for this host (when the
zig_ornament sources are present).  Everything is compared bit-for-bit."""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle_lib as ol
from zig_ornament_gb300 import ornament, scenes

W, H = 96, 64


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def _unit(oracle, fn, a, out_shape):
    f = getattr(oracle.lib, fn)
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_size_t, C.c_void_p]
    a = np.ascontiguousarray(a, np.float32)
    out = np.zeros(out_shape, np.float32)
    f(a.ctypes.data, len(a), out.ctypes.data)
    return out


def test_pcg_sequence(golden, oracle):
    lib = oracle.lib
    lib.oracle_pcg.restype = C.c_int
    lib.oracle_pcg.argtypes = [C.c_uint32, C.c_size_t, C.c_void_p, C.c_void_p]
    for i, seed in enumerate(golden["pcg_seeds"]):
        u = np.zeros(64, np.uint32)
        f = np.zeros(64, np.float32)
        lib.oracle_pcg(int(seed), 64, u.ctypes.data, f.ctypes.data)
        assert np.array_equal(u, golden["pcg_u32"][i])
        assert np.array_equal(bits(f), bits(golden["pcg_f32"][i]))


def test_pcg_python_restatement(golden):
    # random.hip.h:14-30 restated with numpy integer arithmetic
    for i, seed in enumerate(golden["pcg_seeds"]):
        s = np.uint64(seed)
        for k in range(16):
            old = (s + np.uint64(747796405) + np.uint64(2891336453)) & np.uint64(0xFFFFFFFF)
            word = (((old >> ((old >> np.uint64(28)) + np.uint64(4))) ^ old) * np.uint64(277803737)) & np.uint64(0xFFFFFFFF)
            s = (word >> np.uint64(22)) ^ word
            assert int(s) == int(golden["pcg_u32"][i, k])


def test_safe_invdir(golden, oracle):
    out = _unit(oracle, "oracle_safe_invdir", golden["invdir_in"], golden["invdir_out"].shape)
    assert np.array_equal(bits(out), bits(golden["invdir_out"]))


def test_aabb_hit(golden, oracle):
    out = _unit(oracle, "oracle_aabb_hit", golden["aabb_in"], golden["aabb_out"].shape)
    assert np.array_equal(bits(out), bits(golden["aabb_out"]))


def test_triangle_hit(golden, oracle):
    out = _unit(oracle, "oracle_triangle_hit", golden["tri_in"], golden["tri_out"].shape)
    assert np.array_equal(bits(out), bits(golden["tri_out"]))


def test_sphere_hit(golden, oracle):
    out = _unit(oracle, "oracle_sphere_hit", golden["sphere_in"], golden["sphere_out"].shape)
    assert np.array_equal(bits(out), bits(golden["sphere_out"]))


def test_node_count_formulas(golden):
    # src/bvh.zig:17-21,74-75: TLAS = 2*shapes-1, BLAS = sum(2*tris-1)
    spheres, meshes, instances, tris = golden["scene_counts"]
    assert len(golden["scene_tlas_nodes"]) == 2 * (spheres + meshes + instances) - 1
    assert len(golden["scene_blas_nodes"]) == 2 * tris - meshes


def test_trace_rays_golden(golden, golden_bvh, oracle):
    hits, visits = oracle.trace_rays(golden_bvh, golden["rays"])
    ref = golden["ray_hits"]
    assert np.array_equal(hits.view(np.uint32), ref.view(np.uint32))
    assert visits.min() >= 1


def _cases(golden):
    for c in golden["render_cases"]:
        name, spp, ci, depth, gamma, flip, base = str(c).split("|")
        yield name, int(spp), float(ci), int(depth), float(gamma), bool(int(flip)), base or None


@pytest.mark.parametrize("math_name", ["libm", "pmath"])
def test_render_golden(golden, golden_bvh, golden_camera, oracle, math_name):
    states = {}
    for name, spp, ci, depth, gamma, flip, base in _cases(golden):
        cp = ol.make_params(golden_camera, W, H, depth=depth, flip_y=flip, gamma=gamma,
                            textures_count=golden_bvh.scene_textures_count)
        acc0, rng0 = states[base] if base else (None, None)
        acc, rng, fb, _ = oracle.render(golden_bvh, cp, spp, ci_start=ci, acc=acc0, rng=rng0,
                                        portable_math=(math_name == "pmath"))
        states[name] = (acc, rng)
        key = f"render_{math_name}_{name}"
        assert np.array_equal(rng, golden[key + "_rng"]), name
        assert np.array_equal(bits(acc), bits(golden[key + "_acc"])), name
        assert np.array_equal(bits(fb), bits(reference_fb(golden[key + "_fb"], flip))), name


def reference_fb(fb, flip):
    """The reference writes `framebuffer[fb_index] = post_processing(&fb_index, ...)`
    (pathtracer.hip.cpp:25,53): the flipped row only lands in the flipped slot if
    the call is sequenced before the subscript (C++17 assignment order, as clang
    does, and as the WGSL shader spells out, pathtracer.wgsl:87-92).  g++ 13
    reads the subscript first, so the host build of the reference never flips;
    flipping its rows gives the intended result."""
    return fb.reshape(H, -1, 4)[::-1].reshape(-1, 4) if flip else fb


def test_pixel_range_and_threads_do_not_change_results(golden_bvh, golden_camera, oracle):
    cp = ol.make_params(golden_camera, W, H, depth=8, gamma=2.2, textures_count=golden_bvh.scene_textures_count)
    a1, r1, f1, _ = oracle.render(golden_bvh, cp, 3, threads=1)
    a2, r2, f2, _ = oracle.render(golden_bvh, cp, 3, threads=4)
    assert np.array_equal(bits(a1), bits(a2)) and np.array_equal(r1, r2)
    a3, r3, _, _ = oracle.render(golden_bvh, cp, 3, pixel_range=(100, 900))
    assert np.array_equal(bits(a3[100:900]), bits(a1[100:900]))
    assert np.array_equal(r3[:100], np.arange(100, dtype=np.uint32))


def test_fp64_accumulation_matches_fp32_sums(golden_bvh, golden_camera, oracle):
    cp = ol.make_params(golden_camera, W, H, depth=8, textures_count=golden_bvh.scene_textures_count)
    acc64 = np.zeros((W * H, 4), np.float64)
    a, _, _, _ = oracle.render(golden_bvh, cp, 4, acc64=acc64)
    assert np.allclose(acc64, a, rtol=1e-5, atol=1e-5)
    assert (acc64[:, 3] == 4).all()


needs_reference = pytest.mark.skipif(not ol.reference_available(), reason="zig_ornament sources not present")


@needs_reference
@pytest.mark.parametrize("portable", [False, True])
@pytest.mark.parametrize("which", ["spheres", "instanced"])
def test_oracle_matches_compiled_reference(which, portable, oracle):
    """Live pin: a different scene from the fixture, rendered by the
    reference's own kernels and by the restatement."""
    if which == "spheres":
        scene, w, h, depth = scenes.spheres_scene(64, 36, seed=3), 64, 36, 10
    else:
        scene = scenes.instanced_meshes_scene(80, 45, seed=5, n_blas=3, n_instances=12, tri_range=(200, 2000),
                                              texture_size=64, box=12.0)
        w, h, depth = 80, 45, 8
    bvh = ornament.Bvh(scene)
    ref = ol.Reference(portable_math=portable)
    cp = ol.make_params(scene.camera, w, h, depth=depth, gamma=2.2, textures_count=bvh.scene_textures_count)
    ra, rr, rf = ref.render(bvh, cp, 3)
    cp_flip = ol.make_params(scene.camera, w, h, depth=depth, gamma=2.2, flip_y=True,
                             textures_count=bvh.scene_textures_count)
    _, _, rf_flip = ref.render(bvh, cp_flip, 3)
    assert np.array_equal(bits(rf_flip), bits(rf))   # the g++ build does not flip (see reference_fb)
    _, _, of_flip, _ = oracle.render(bvh, cp_flip, 3, portable_math=portable)
    assert np.array_equal(bits(of_flip), bits(rf.reshape(h, w, 4)[::-1].reshape(-1, 4)))
    oa, orr, of, _ = oracle.render(bvh, cp, 3, portable_math=portable)
    assert np.array_equal(rr, orr)
    assert np.array_equal(bits(ra), bits(oa))
    assert np.array_equal(bits(rf), bits(of))
    rs = np.random.default_rng(11)
    rays = np.concatenate([rs.uniform(-20, 20, (2000, 3)), rs.normal(size=(2000, 3))], 1).astype(np.float32)
    assert np.array_equal(ref.trace_rays(bvh, rays).view(np.uint32), oracle.trace_rays(bvh, rays)[0].view(np.uint32))


@needs_reference
def test_reference_struct_layouts():
    sizes = ol.Reference().struct_sizes()
    assert sizes == {"BvhNode": 64, "Material": 32, "ConstantParams": 144, "Camera": 112, "float4x4": 64}
