"""GPU parity: the sm_103a kernels through the C ABI against the reference
(golden vectors recorded from its own HIP kernels) and the CPU oracle.

Bit-exact throughout: hits, t values, node-visit counts, accumulation
buffers, RNG states and framebuffers are compared as raw 32-bit words.  The
kernels use the project's portable transcendentals, so images match the
reference built with the same transcendentals ("pmath" fixtures) exactly."""
import numpy as np
import pytest

from oracle import oracle_lib as ol
from zig_ornament_gb300 import _lib, ornament, scenes

pytestmark = pytest.mark.gpu

W, H = 96, 64


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


KERNELS = [_lib.KERNEL_MEGA, _lib.KERNEL_WAVEFRONT]
KERNEL_IDS = ["mega", "wavefront"]


def make_state(depth=8, gamma=1.0, flip=False, iterations=1, semantics=_lib.SEMANTICS_HIP, spp_per_launch=0,
               eps=0.001, kernel=_lib.KERNEL_MEGA):
    s = _lib.State()
    s.depth, s.flip_y = depth, 1 if flip else 0
    s.inverted_gamma = float(np.float32(1.0) / np.float32(gamma))
    s.iterations, s.ray_cast_epsilon = iterations, eps
    s.semantics, s.kernel, s.spp_per_launch = semantics, kernel, spp_per_launch
    return s


@pytest.fixture(scope="module")
def golden_renderer(golden_bvh):
    r = ornament.Renderer(golden_bvh, device=0)
    yield r
    r.close()


def test_trace_rays_matches_reference_and_oracle(golden, golden_bvh, golden_renderer, oracle):
    golden_renderer.set_state(make_state())
    hits, visits = golden_renderer.trace_rays(golden["rays"])
    assert np.array_equal(bits(hits), bits(golden["ray_hits"]))       # reference's Bvh::hit
    _, ovisits = oracle.trace_rays(golden_bvh, golden["rays"])
    assert np.array_equal(visits, ovisits)                              # per-ray node visits


def test_trace_rays_exact_slab_fallback(golden_bvh, golden_renderer, oracle):
    """Rays whose origins are NaN, infinite or beyond 1e30 take the
    reference's own RT_MIN/RT_MAX slab form; all others the FMNMX form.
    Both must give the reference's hits and visit counts."""
    rs = np.random.default_rng(3)
    rays = np.concatenate([rs.uniform(-3, 3, (512, 3)), rs.normal(size=(512, 3))], 1).astype(np.float32)
    rays[0:8, 0] = np.nan
    rays[8:16, 1] = np.inf
    rays[16:24, 2] = -3e30
    rays[24:32, 3:6] = 0.0                      # zero direction: safe_invdir clamps
    rays[32:40, 3] = np.nan                     # NaN direction
    rays[40:48, 0:3] = 1e29                     # large but below the guard
    golden_renderer.set_state(make_state())
    hits, visits = golden_renderer.trace_rays(rays)
    ohits, ovisits = oracle.trace_rays(golden_bvh, rays)
    assert np.array_equal(bits(hits), bits(ohits))
    assert np.array_equal(visits, ovisits)


def _golden_cases(golden):
    for c in golden["render_cases"]:
        name, spp, ci, depth, gamma, flip, base = str(c).split("|")
        yield name, int(spp), float(ci), int(depth), float(gamma), bool(int(flip)), base or None


def _flip_rows(fb, flip):
    # the host build of the reference never flips (see tests/test_oracle_golden.py::reference_fb)
    return fb.reshape(H, -1, 4)[::-1].reshape(-1, 4) if flip else fb


@pytest.mark.parametrize("kernel", KERNELS, ids=KERNEL_IDS)
def test_render_matches_reference_pmath(golden, golden_camera, golden_renderer, kernel):
    """PathTracer.render semantics end to end: the fused single pass, a
    multi-pass render, a continued (progressive) render, flip_y + gamma."""
    r = golden_renderer
    r.set_resolution(W, H)
    states = {}
    for name, spp, ci, depth, gamma, flip, base in _golden_cases(golden):
        r.set_resolution(W, H)          # fresh target: RNG reseeded with the pixel index
        r.set_state(make_state(depth=depth, gamma=gamma, flip=flip, iterations=spp, kernel=kernel))
        r.set_camera(golden_camera)
        if base:
            acc0, rng0 = states[base]
            r.set_progress(acc0, rng0, ci - 1.0)
        r.render()
        acc, rng, cur = r.progress()
        fb = r.framebuffer()
        states[name] = (acc, rng)
        key = f"render_pmath_{name}"
        assert cur == ci + spp - 1
        assert np.array_equal(rng, golden[key + "_rng"]), name
        assert np.array_equal(bits(acc), bits(golden[key + "_acc"])), name
        assert np.array_equal(bits(fb), bits(_flip_rows(golden[key + "_fb"], flip))), name


@pytest.mark.parametrize("kernel", KERNELS, ids=KERNEL_IDS)
@pytest.mark.parametrize("spp_per_launch", [1, 2, 7])
def test_launch_chunking_does_not_change_results(golden_camera, golden_renderer, golden, spp_per_launch, kernel):
    r = golden_renderer
    r.set_resolution(W, H)
    r.set_state(make_state(gamma=2.2, iterations=5, spp_per_launch=spp_per_launch, kernel=kernel))
    r.set_camera(golden_camera)
    r.render()
    acc, rng, _ = r.progress()
    assert np.array_equal(bits(acc), bits(golden["render_pmath_pass5_acc"]))
    assert np.array_equal(rng, golden["render_pmath_pass5_rng"])


@pytest.mark.parametrize("kernel", KERNELS, ids=KERNEL_IDS)
@pytest.mark.parametrize("semantics", [_lib.SEMANTICS_HIP, _lib.SEMANTICS_WGSL])
def test_semantics_vs_oracle(golden_bvh, golden_camera, golden_renderer, oracle, semantics, kernel):
    r = golden_renderer
    r.set_resolution(W, H)
    r.set_state(make_state(depth=10, gamma=2.2, iterations=4, semantics=semantics, kernel=kernel))
    r.set_camera(golden_camera)
    r.render()
    acc, rng, _ = r.progress()
    fb = r.framebuffer()
    cp = ol.make_params(golden_camera, W, H, depth=10, gamma=2.2, textures_count=golden_bvh.scene_textures_count)
    oacc, orng, ofb, _ = oracle.render(golden_bvh, cp, 4, semantics=semantics, portable_math=True)
    assert np.array_equal(rng, orng)
    assert np.array_equal(bits(acc), bits(oacc))
    assert np.array_equal(bits(fb), bits(ofb))


def test_camera_dirty_restarts_accumulation(golden_camera, golden_renderer, golden):
    """update(): a dirty camera resets current_iteration
    (src/hip_backend/path_tracer.zig:150-158); the RNG stream continues."""
    r = golden_renderer
    r.set_resolution(W, H)
    r.set_state(make_state(gamma=2.2, iterations=5))
    r.set_camera(golden_camera)
    r.render()
    _, rng5, _ = r.progress()
    r.set_camera(golden_camera)           # same camera, but dirty
    r.set_state(make_state(gamma=2.2, iterations=1))
    r.render()
    acc, rng, cur = r.progress()
    assert cur == 1.0
    assert (acc[:, 3] == 1.0).all()       # accumulation restarted
    assert not np.array_equal(rng, rng5)  # the RNG stream moved on


def test_set_resolution_reseeds(golden_camera, golden_renderer, golden):
    r = golden_renderer
    r.set_resolution(W, H)
    r.set_state(make_state(gamma=2.2, iterations=5))
    r.set_camera(golden_camera)
    r.render()
    r.set_resolution(W, H)
    r.set_camera(golden_camera)
    r.render()
    acc, rng, _ = r.progress()
    assert np.array_equal(rng, golden["render_pmath_pass5_rng"])


def test_errors_are_statuses(golden_bvh, golden_renderer):
    r = golden_renderer
    r.set_resolution(W, H)
    with pytest.raises(_lib.OrnamentError) as e:
        r._check(r._lib.orn_get_framebuffer(r.handle, np.zeros(16, np.float32).ctypes.data, 4))
    assert e.value.status == 8
    fresh = ornament.Renderer(golden_bvh, device=0)
    with pytest.raises(_lib.OrnamentError) as e:
        fresh.render()                     # no camera yet
    assert e.value.status == 1
    fresh.close()
    bad = ornament.Bvh.from_arrays(**{k: getattr(golden_bvh, k) for k in
                                     ("blas_nodes", "normals", "normal_indices", "uvs", "uv_indices",
                                      "transforms", "materials", "textures", "scene_textures_count")},
                                   tlas_nodes=golden_bvh.tlas_nodes.copy())
    bad.tlas_nodes["left_or_custom_id"][-1] = len(bad.tlas_nodes) + 5
    with pytest.raises(_lib.OrnamentError) as e:
        ornament.Renderer(bad, device=0)
    assert e.value.status == 6


def test_pathtracer_surface_end_to_end(oracle):
    """The ornament.zig-style driver loop: State setters, setResolution,
    render, getFrameBuffer, camera move (setLookAt)."""
    scene = scenes.small_test_scene(64, 40, seed=9)
    pt = ornament.PathTracer(scene, device=0)
    pt.state.setGamma(2.2)
    pt.state.setFlipY(True)
    pt.state.setDepth(6)
    pt.state.setIterations(3)
    pt.setResolution(ornament.Resolution(64, 40))
    pt.render()
    fb1 = pt.getFrameBuffer().copy()
    cp = ol.make_params(scene.camera, 64, 40, depth=6, gamma=2.2, flip_y=True,
                        textures_count=pt.bvh.scene_textures_count)
    _, _, ofb, _ = oracle.render(pt.bvh, cp, 3)
    assert np.array_equal(bits(fb1), bits(ofb))
    scene.camera.setLookAt(ornament.f32x4(1, 3, 12, 1), ornament.f32x4(0, 0.5, 0, 1), ornament.f32x4(0, 1, 0, 0))
    pt.render()
    fb2 = pt.getFrameBuffer()
    assert not np.array_equal(fb1, fb2)
    _, _, ci = pt.getProgress()
    assert ci == 3.0
    pt.deinit()


@pytest.mark.parametrize("kernel", KERNELS, ids=KERNEL_IDS)
def test_sphere_field_and_instanced_vs_oracle(oracle, kernel):
    for scene, w, h, depth in ((scenes.spheres_scene(80, 45, seed=0), 80, 45, 10),
                               (scenes.instanced_meshes_scene(96, 54, seed=1, n_blas=4, n_instances=40,
                                                              tri_range=(2000, 8000), texture_size=128), 96, 54, 8)):
        bvh = ornament.Bvh(scene)
        r = ornament.Renderer(bvh, device=0)
        r.set_resolution(w, h)
        r.set_state(make_state(depth=depth, gamma=2.2, iterations=2, kernel=kernel))
        r.set_camera(scene.camera.to_struct())
        r.render()
        acc, rng, _ = r.progress()
        cp = ol.make_params(scene.camera, w, h, depth=depth, gamma=2.2, textures_count=bvh.scene_textures_count)
        oacc, orng, _, _ = oracle.render(bvh, cp, 2)
        assert np.array_equal(rng, orng)
        assert np.array_equal(bits(acc), bits(oacc))
        r.close()


def _primary_rays(cam, w, h, n, rs):
    """Camera rays (camera.hip.h:25-33 formula, float32) at random pixels."""
    px = rs.integers(0, w, n)
    py = rs.integers(0, h, n)
    u = ((px + rs.random(n)) / (w - 1)).astype(np.float32)[:, None]
    v = ((py + rs.random(n)) / (h - 1)).astype(np.float32)[:, None]
    o = np.array(cam.origin[:], np.float32)
    d = (np.array(cam.lower_left_corner[:], np.float32) + u * np.array(cam.horizontal[:], np.float32)
         + v * np.array(cam.vertical[:], np.float32) - o)
    return np.concatenate([np.broadcast_to(o, d.shape), d], 1).astype(np.float32)


def test_primary_hits_instanced_1080p_scene(oracle):
    """The benchmark scene (8 BLAS, 256 instances, 281k triangles): primary
    hit instance/primitive ids, t and node-visit counts, bit-exact."""
    scene = scenes.instanced_meshes_scene()
    bvh = ornament.Bvh(scene)
    r = ornament.Renderer(bvh, device=0)
    r.set_state(make_state())
    rays = _primary_rays(scene.camera.to_struct(), 1920, 1080, 200_000, np.random.default_rng(5))
    hits, visits = r.trace_rays(rays)
    ohits, ovisits = oracle.trace_rays(bvh, rays)
    assert np.array_equal(bits(hits), bits(ohits))
    assert np.array_equal(visits, ovisits)
    assert hits["hit"].mean() > 0.05
    r.close()


@pytest.mark.parametrize("kernel", KERNELS, ids=KERNEL_IDS)
def test_depth_zero_and_one(golden_bvh, golden_camera, golden_renderer, oracle, kernel):
    """Edge cases of the bounce loop: depth 0 (no ray at all: every sample is
    white) and depth 1 (camera rays only)."""
    r = golden_renderer
    for depth in (0, 1):
        r.set_resolution(W, H)
        r.set_state(make_state(depth=depth, iterations=3, kernel=kernel))
        r.set_camera(golden_camera)
        r.render()
        acc, rng, _ = r.progress()
        cp = ol.make_params(golden_camera, W, H, depth=depth, textures_count=golden_bvh.scene_textures_count)
        oacc, orng, _, _ = oracle.render(golden_bvh, cp, 3)
        assert np.array_equal(rng, orng) and np.array_equal(bits(acc), bits(oacc)), depth
        if depth == 0:
            assert (acc == 3.0).all()     # three white samples, alpha 3


def test_kernels_agree_at_1080p():
    """Megakernel and wavefront give the same bits on the benchmark scene."""
    scene = scenes.instanced_meshes_scene()
    bvh = ornament.Bvh(scene)
    out = []
    for kernel in KERNELS:
        r = ornament.Renderer(bvh, device=0)
        r.set_resolution(1920, 1080)
        r.set_state(make_state(iterations=2, kernel=kernel))
        r.set_camera(scene.camera.to_struct())
        r.render()
        out.append(r.progress())
        r.close()
    assert np.array_equal(bits(out[0][0]), bits(out[1][0])) and np.array_equal(out[0][1], out[1][1])


@pytest.mark.slow
@pytest.mark.parametrize("kernel", KERNELS, ids=KERNEL_IDS)
def test_full_size_properties_1080p(kernel):
    """Full-size (1920x1080) properties: deterministic, progressive renders
    equal one-shot renders, alpha counts the samples, values finite, work
    counters consistent."""
    scene = scenes.instanced_meshes_scene()
    bvh = ornament.Bvh(scene)
    a = ornament.Renderer(bvh, device=0)
    b = ornament.Renderer(bvh, device=0)
    for r in (a, b):
        r.set_resolution(1920, 1080)
        r.set_camera(scene.camera.to_struct())
    a.set_state(make_state(iterations=4, kernel=kernel))
    a.enable_counters(True)
    a.render()
    b.set_state(make_state(iterations=2, kernel=kernel))
    b.render()
    b.render()
    acc_a, rng_a, ci_a = a.progress()
    acc_b, rng_b, ci_b = b.progress()
    assert ci_a == ci_b == 4.0
    assert np.array_equal(bits(acc_a), bits(acc_b)) and np.array_equal(rng_a, rng_b)
    assert (acc_a[:, 3] == 4.0).all()
    assert np.isfinite(acc_a).all()
    c = a.counters()
    assert c["samples"] == 4 * 1920 * 1080
    assert c["rays"] >= c["samples"]
    assert c["visits"] == c["internal"] + c["sphere_leaf"] + c["mesh_entry"] + c["triangle"]
    assert c["sphere_hits"] + c["mesh_hits"] <= c["rays"]
    a.close()
    b.close()


def test_large_scene_sampled_pixels_vs_oracle(oracle):
    """Config-4 scale (4096 instances over ~10M triangles, 3840x2160, depth
    16): one pass of the megakernel over the whole frame, every 2003rd pixel
    checked bit for bit against the oracle (accumulation and RNG state)."""
    w, h, stride = 3840, 2160, 2003
    scene = scenes.large_scene(w, h)
    bvh = ornament.Bvh(scene)
    r = ornament.Renderer(bvh, device=0)
    r.set_resolution(w, h)
    r.set_state(make_state(depth=16, iterations=1))
    r.set_camera(scene.camera.to_struct())
    r.render()
    acc, rng, _ = r.progress()
    cp = ol.make_params(scene.camera, w, h, depth=16, textures_count=bvh.scene_textures_count)
    oacc, orng, _, _ = oracle.render(bvh, cp, 1, pixel_range=(0, w * h), pixel_stride=stride)
    idx = np.arange(0, w * h, stride)
    assert len(idx) > 4000
    assert np.array_equal(rng[idx], orng[idx])
    assert np.array_equal(bits(acc[idx]), bits(oacc[idx]))
    r.close()


@pytest.mark.parametrize("kernel", KERNELS, ids=KERNEL_IDS)
def test_sah_tree_renders_like_the_oracle(oracle, kernel):
    """The non-parity SAH tree runs through the same kernels: bit for bit
    what the oracle's traversal gives on that tree."""
    scene = scenes.instanced_meshes_scene(96, 54, seed=1, n_blas=4, n_instances=40, tri_range=(2000, 8000),
                                          texture_size=128)
    bvh = ornament.Bvh(scene, builder="sah")
    r = ornament.Renderer(bvh, device=0)
    r.set_resolution(96, 54)
    r.set_state(make_state(depth=8, gamma=2.2, iterations=2, kernel=kernel))
    r.set_camera(scene.camera.to_struct())
    r.render()
    acc, rng, _ = r.progress()
    cp = ol.make_params(scene.camera, 96, 54, depth=8, gamma=2.2, textures_count=bvh.scene_textures_count)
    oacc, orng, _, _ = oracle.render(bvh, cp, 2)
    assert np.array_equal(rng, orng)
    assert np.array_equal(bits(acc), bits(oacc))
    r.close()


@pytest.mark.parametrize("kernel", [_lib.KERNEL_MEGA, _lib.KERNEL_WAVEFRONT, _lib.KERNEL_CACHED,
                                    _lib.KERNEL_CACHED_WAVEFRONT],
                         ids=["mega", "wavefront", "cached", "cached-wavefront"])
def test_pixel_order_does_not_change_results(kernel):
    """Longest-first hand-out (orn_state.pixel_order = COST, the default)
    against raster order over several launches: the same bits."""
    scene = scenes.instanced_meshes_scene(96, 54, seed=1, n_blas=4, n_instances=40, tri_range=(2000, 8000),
                                          texture_size=64, n_lights=3)
    bvh = ornament.Bvh(scene)
    outs = []
    for order in (_lib.PIXEL_ORDER_RASTER, _lib.PIXEL_ORDER_COST):
        r = ornament.Renderer(bvh, device=0)
        cache = None
        if kernel in (_lib.KERNEL_CACHED, _lib.KERNEL_CACHED_WAVEFRONT):
            # no training steps: float atomics in the weight-gradient sums
            # make trained weights differ in the last bits between runs
            cache = ornament.RadianceCache(seed=1, train_shift=3, steps_per_frame=0)
            r.attach_cache(cache)
        r.set_resolution(96, 54)
        # (for the cached kernel spp_per_launch counts sample streams, whose
        # atomic accumulation is not bit-reproducible: one stream there)
        st = make_state(depth=8, iterations=6, spp_per_launch=2 if kernel == _lib.KERNEL_MEGA else 0,
                        kernel=kernel)
        st.pixel_order = order
        r.set_state(st)
        r.set_camera(scene.camera.to_struct())
        r.render()
        r.render()
        acc, rng, _ = r.progress()
        outs.append((bits(acc), rng))
        r.close()
        if cache is not None:
            cache.close()
    assert np.array_equal(outs[0][0], outs[1][0])
    assert np.array_equal(outs[0][1], outs[1][1])
