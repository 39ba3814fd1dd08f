"""Radiance cache on the GPU: the tensor-core MLP against the FP64 oracle
(forward, gradients, Adam), training convergence, and the cached renderer's
gain over plain tracing at equal time."""
import numpy as np
import pytest

from oracle import radiance_cache as rco
from zig_ornament_gb300 import _lib, ornament, scenes

pytestmark = pytest.mark.gpu


def _layer_errors(g, ref):
    out = []
    for l in range(6):
        a, b = g[rco.OFFSETS[l]:rco.OFFSETS[l + 1]], ref[rco.OFFSETS[l]:rco.OFFSETS[l + 1]]
        out.append(float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)))
    return out


def _samples(n, seed):
    rng = np.random.default_rng(seed)
    x = rng.uniform(0, 1, size=(n, 10)).astype(np.float32)
    t = rng.uniform(0, 2, size=(n, 3)).astype(np.float32)
    t[::9, 0] = -1.0   # samples without a target
    return x, t


def test_forward_matches_oracle():
    cache = ornament.RadianceCache(seed=11)
    p = cache.params()
    x, _ = _samples(1000, 1)   # not a multiple of the 128-row tile
    y = cache.infer(x).astype(np.float64)
    y_em, _, _ = rco.forward(p, x, emulate=True)
    y_ex, _, _ = rco.forward(p, x)
    e_em = np.linalg.norm(y - y_em) / np.linalg.norm(y_em)
    e_ex = np.linalg.norm(y - y_ex) / np.linalg.norm(y_ex)
    print(f"forward rel. L2 error: {e_em:.2e} vs emulated, {e_ex:.2e} vs FP64")
    assert e_em < 5e-3
    assert e_ex < 2e-2
    cache.close()


def test_gradients_match_oracle():
    cache = ornament.RadianceCache(seed=12)
    p = cache.params()
    x, t = _samples(777, 2)
    g, loss = cache.gradients(x, t)
    l_em, g_em = rco.loss_and_grads(p, x, t, emulate=True)
    l_ex, g_ex = rco.loss_and_grads(p, x, t)
    e_em, e_ex = _layer_errors(g, g_em), _layer_errors(g, g_ex)
    print("per-layer gradient rel. L2 error vs emulated:", ["%.1e" % e for e in e_em])
    print("per-layer gradient rel. L2 error vs FP64:    ", ["%.1e" % e for e in e_ex])
    assert loss == pytest.approx(l_ex, rel=2e-2)
    assert max(e_em) < 2e-2
    assert max(e_ex) < 6e-2
    cos = float(g @ g_ex / (np.linalg.norm(g) * np.linalg.norm(g_ex)))
    assert cos > 0.998
    # the weights did not move
    assert np.array_equal(cache.params(), p)
    cache.close()


def test_adam_step_matches_oracle():
    cache = ornament.RadianceCache(seed=13)
    p0 = cache.params()
    x, t = _samples(512, 3)
    g, _ = cache.gradients(x, t)
    cache.train(x, t)
    p1 = cache.params().astype(np.float64)
    expect, _, _ = rco.adam_step(p0.astype(np.float64), 0.0, 0.0, g, step=1, grad_scale=1.0 / (3 * len(x)))
    real = np.ones(rco.PARAM_COUNT, bool)
    real[rco.OFFSETS[5] + 3 * 64:] = False
    big = real & (np.abs(g) / (3 * len(x)) > 1e-6)
    assert big.sum() > 10000
    assert np.allclose(p1[big], expect[big], rtol=0, atol=2e-6)
    assert not p1[~real].any()
    cache.close()


def test_training_fits_a_smooth_function():
    cache = ornament.RadianceCache(seed=14)
    rng = np.random.default_rng(4)

    def target(x):
        return np.stack([0.6 + 0.4 * np.sin(2 * np.pi * x[:, 0]) * x[:, 9],
                         0.3 + 0.2 * x[:, 1] * x[:, 4],
                         0.5 + 0.3 * np.cos(3 * x[:, 2] + x[:, 7])], axis=1).astype(np.float32)

    xv = rng.uniform(0, 1, size=(4096, 10)).astype(np.float32)
    tv = target(xv)

    def val_loss():
        y = cache.infer(xv)
        return float(np.mean((y - tv) ** 2 / (y.astype(np.float64) ** 2 + 0.01)))

    before = val_loss()
    for _ in range(300):
        x = rng.uniform(0, 1, size=(4096, 10)).astype(np.float32)
        cache.train(x, target(x))
    after = val_loss()
    print(f"validation relative L2: {before:.3e} -> {after:.3e}")
    assert after < 0.03 * before
    assert after < 0.1
    assert cache.stats()["steps"] == 300
    cache.close()


def _cache_scene(w, h):
    return scenes.instanced_meshes_scene(w, h, seed=5, n_blas=4, n_instances=96, tri_range=(4_000, 20_000),
                                         n_textures=2, texture_size=256, n_lights=3)


def _renderer(scene, w, h, kernel):
    bvh = ornament.Bvh(scene, row_major_transforms=True)
    r = ornament.Renderer(bvh, 0)
    r.set_resolution(w, h)
    st = ornament.State()
    st.depth = 8
    st.kernel = kernel
    r.set_state(st.to_struct())
    r.set_camera(scene.camera.to_struct())
    return r, st


def test_cached_render_runs_and_trains():
    w, h = 160, 96
    scene = _cache_scene(w, h)
    r, st = _renderer(scene, w, h, _lib.KERNEL_CACHED)
    cache = ornament.RadianceCache(seed=1, batch=2048)
    r.attach_cache(cache)
    st.iterations = 8
    r.set_state(st.to_struct())
    r.render()
    r.synchronize()
    acc = r.accumulation()
    assert np.isfinite(acc).all()
    assert np.all(acc[:, 3] == 8)
    s = cache.stats()
    assert s["frames"] == 8 and s["steps"] > 0
    fb = r.framebuffer()
    assert np.isfinite(fb).all() and fb[:, :3].max() > 0
    # kernel CACHED without a cache is refused
    r.attach_cache(None)
    with pytest.raises(_lib.OrnamentError):
        r.render()
    r.close()
    cache.close()


def _run_for(r, st, scene, frames):
    r.set_camera(scene.camera.to_struct())   # restart the accumulation
    st.iterations = frames
    r.set_state(st.to_struct())
    r.render()
    return r.last_render_ms()


def test_cache_gains_at_equal_time():
    """What the trained network gains: relMSE against a 16k-spp FP64 render
    of a closed room (long multi-bounce paths) after the same GPU time, for
    the cached renderer (its warm-up training frames included in its time),
    the same renderer without the network (every pixel traces its full path
    with the same light sampling: unbiased), and plain megakernel tracing."""
    w, h = 320, 180
    scene = scenes.cornell_box_scene(w, h)
    ref_r, _ = _renderer(scene, w, h, _lib.KERNEL_MEGA)
    ref = ref_r.render_f64(16384)
    ref_r.close()

    rc, stc = _renderer(scene, w, h, _lib.KERNEL_CACHED)
    cache = ornament.RadianceCache(seed=1, train_shift=3)
    rc.attach_cache(cache)
    t_cached = _run_for(rc, stc, scene, 64)           # warm-up training
    t_cached += _run_for(rc, stc, scene, 192)
    e_cached, skip_c = rc.relmse(ref, return_skipped=True)
    rc.attach_cache(None)
    cache.close()

    def equal_time(kernel, **cfg):
        r, st = _renderer(scene, w, h, kernel)
        c = None
        if cfg:
            c = ornament.RadianceCache(seed=1, **cfg)
            r.attach_cache(c)
        ms = _run_for(r, st, scene, 16) / 16
        n = max(1, int(t_cached / ms))
        t = _run_for(r, st, scene, n)
        e = r.relmse(ref)
        r.close()
        if c is not None:
            c.close()
        return n, t, e

    n_nee, t_nee, e_nee = equal_time(_lib.KERNEL_CACHED, train_shift=0, steps_per_frame=0)
    n_plain, t_plain, e_plain = equal_time(_lib.KERNEL_MEGA)
    print(f"equal time {t_cached:.1f} ms: cached relMSE {e_cached:.3e} (256 frames incl. 64 warm-up); "
          f"without the network {e_nee:.3e} ({n_nee} frames, {t_nee:.1f} ms); "
          f"plain {e_plain:.3e} ({n_plain} spp, {t_plain:.1f} ms); "
          f"gain {e_nee / e_cached:.2f}x over no network, {e_plain / e_cached:.2f}x over plain")
    assert skip_c <= 4
    assert t_nee <= 1.15 * t_cached and t_plain <= 1.15 * t_cached
    assert e_cached < e_nee
    assert e_cached < e_plain
    rc.close()


def test_light_sampling_is_unbiased():
    """The cached renderer without the network (every pixel a training pixel)
    estimates the reference's image: its mean matches a plain FP64 render."""
    w, h = 160, 96
    scene = _cache_scene(w, h)
    ref_r, _ = _renderer(scene, w, h, _lib.KERNEL_MEGA)
    ref = ref_r.render_f64(8192)
    ref_r.close()
    r, st = _renderer(scene, w, h, _lib.KERNEL_CACHED)
    cache = ornament.RadianceCache(seed=1, train_shift=0, steps_per_frame=0)
    r.attach_cache(cache)
    _run_for(r, st, scene, 1024)
    acc = r.accumulation().astype(np.float64)
    m = acc[:, :3] / acc[:, 3:4]
    ok = np.isfinite(m).all(axis=1) & np.isfinite(ref[:, :3]).all(axis=1)
    mean_nee, mean_ref = m[ok].mean(axis=0), ref[ok, :3].mean(axis=0)
    print("image mean: light sampling", mean_nee.round(5), "reference", mean_ref.round(5))
    assert np.allclose(mean_nee, mean_ref, rtol=3e-3)
    e = r.relmse(ref)
    r.close()
    cache.close()
    assert e < 5e-3


def test_sample_streams():
    """Several sample streams per pixel in one cached launch
    (orn_state.spp_per_launch = 4): every pixel gets frames x 4 samples, and
    without the network (every pixel traces full paths) the image mean still
    matches a plain FP64 render."""
    w, h = 160, 96
    scene = _cache_scene(w, h)
    r, st = _renderer(scene, w, h, _lib.KERNEL_CACHED)
    st.spp_per_launch = 4
    cache = ornament.RadianceCache(seed=1, batch=2048)
    r.attach_cache(cache)
    _run_for(r, st, scene, 8)
    acc = r.accumulation()
    assert np.isfinite(acc).all()
    assert np.all(acc[:, 3] == 32)
    assert cache.stats()["frames"] == 8
    fb = r.framebuffer()
    assert np.isfinite(fb).all() and fb[:, :3].max() > 0
    r.attach_cache(None)
    r.close()
    cache.close()

    ref_r, _ = _renderer(scene, w, h, _lib.KERNEL_MEGA)
    ref = ref_r.render_f64(8192)
    ref_r.close()
    r, st = _renderer(scene, w, h, _lib.KERNEL_CACHED)
    st.spp_per_launch = 4
    cache = ornament.RadianceCache(seed=1, train_shift=0, steps_per_frame=0)
    r.attach_cache(cache)
    _run_for(r, st, scene, 256)
    acc = r.accumulation().astype(np.float64)
    assert np.all(acc[:, 3] == 1024)
    m = acc[:, :3] / acc[:, 3:4]
    ok = np.isfinite(m).all(axis=1) & np.isfinite(ref[:, :3]).all(axis=1)
    mean_s, mean_ref = m[ok].mean(axis=0), ref[ok, :3].mean(axis=0)
    print("image mean: 4 streams", mean_s.round(5), "reference", mean_ref.round(5))
    assert np.allclose(mean_s, mean_ref, rtol=3e-3)
    assert r.relmse(ref) < 5e-3
    r.close()
    cache.close()


def test_sobol_sampler_is_unbiased():
    """The cached renderer's Owen-scrambled Sobol sampler
    (orn_state.sampler = SOBOL) without the network: the image mean matches
    a plain FP64 render, and at equal samples its error is below the PCG
    stream's."""
    w, h = 160, 96
    scene = _cache_scene(w, h)
    ref_r, _ = _renderer(scene, w, h, _lib.KERNEL_MEGA)
    ref = ref_r.render_f64(8192)
    ref_r.close()
    errs = {}
    for sampler in (_lib.SAMPLER_PCG, _lib.SAMPLER_SOBOL):
        r, st = _renderer(scene, w, h, _lib.KERNEL_CACHED)
        st.spp_per_launch = 4
        st.sampler = sampler
        cache = ornament.RadianceCache(seed=1, train_shift=0, steps_per_frame=0)
        r.attach_cache(cache)
        _run_for(r, st, scene, 64)
        acc = r.accumulation().astype(np.float64)
        m = acc[:, :3] / acc[:, 3:4]
        ok = np.isfinite(m).all(axis=1) & np.isfinite(ref[:, :3]).all(axis=1)
        mean_s, mean_ref = m[ok].mean(axis=0), ref[ok, :3].mean(axis=0)
        errs[sampler] = r.relmse(ref)
        print("sampler", sampler, "image mean", mean_s.round(5), "reference", mean_ref.round(5),
              "relMSE at 256 spp", errs[sampler])
        assert np.allclose(mean_s, mean_ref, rtol=5e-3)
        r.close()
        cache.close()
    assert errs[_lib.SAMPLER_SOBOL] < errs[_lib.SAMPLER_PCG]


@pytest.mark.parametrize("sampler", [_lib.SAMPLER_PCG, _lib.SAMPLER_SOBOL], ids=["pcg", "sobol"])
@pytest.mark.parametrize("semantics", [_lib.SEMANTICS_HIP, _lib.SEMANTICS_WGSL], ids=["hip", "wgsl"])
def test_cached_wavefront_matches_cached_megakernel(sampler, semantics):
    """The cached renderer on the persistent wavefront (KERNEL_CACHED_WAVEFRONT)
    runs the cached megakernel's path logic (KERNEL_CACHED) operation for
    operation: with the network's part off (every path a training path,
    train_shift 0, no training steps) and one sample stream, both give the
    same accumulation and RNG states bit for bit over several frames —
    light sampling, shadow rays, cache-vertex records and all."""
    w, h = 160, 96
    scene = _cache_scene(w, h)
    out = {}
    for kernel in (_lib.KERNEL_CACHED, _lib.KERNEL_CACHED_WAVEFRONT):
        r, st = _renderer(scene, w, h, kernel)
        st.sampler = sampler
        st.semantics = semantics
        cache = ornament.RadianceCache(seed=1, train_shift=0, steps_per_frame=0)
        r.attach_cache(cache)
        _run_for(r, st, scene, 6)
        acc, rng, ci = r.progress()
        out[kernel] = (np.ascontiguousarray(acc).view(np.uint32).copy(), rng.copy(), ci)
        r.synchronize()
        r.attach_cache(None)
        r.close()
        cache.close()
    a, b = out[_lib.KERNEL_CACHED], out[_lib.KERNEL_CACHED_WAVEFRONT]
    assert a[2] == b[2] == 6.0
    assert np.array_equal(a[1], b[1])
    assert np.array_equal(a[0], b[0])
