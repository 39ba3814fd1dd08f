"""GPU: the tcgen05 GEMM encodings used by the radiance cache, and the FP64
16k-spp-style oracle render with its FP64 relMSE reduction."""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle_lib as ol
from zig_ornament_gb300 import _lib, ornament, scenes

pytestmark = pytest.mark.gpu


def to16(x, bf16):
    x = np.asarray(x, np.float32)
    if bf16:
        u = x.view(np.uint32)
        u = (u + 0x7FFF + ((u >> 16) & 1)) >> 16          # round to nearest even
        return u.astype(np.uint16), (u.astype(np.uint32) << 16).view(np.float32)
    h = x.astype(np.float16)
    return h.view(np.uint16), h.astype(np.float32)


@pytest.mark.parametrize("mn_major", [False, True])
@pytest.mark.parametrize("bf16", [False, True])
@pytest.mark.parametrize("K,N", [(16, 16), (64, 64), (256, 64), (64, 128), (256, 16), (128, 64), (128, 16)])
def test_tcgen05_gemm_matches_host(K, N, bf16, mn_major):
    lib = _lib.load()
    rs = np.random.default_rng(K * 1000 + N + bf16)
    a16, a = to16(rs.normal(size=(128, K)), bf16)
    b16, b = to16(rs.normal(size=(N, K)), bf16)
    d = np.zeros((128, N), np.float32)
    mode = 2 if mn_major else 0
    st = lib.orn_tc_selftest(K, N, int(bf16), mode, a16.ctypes.data, b16.ctypes.data, d.ctypes.data)
    assert st == 0, lib.orn_status_string(st)
    ref = a.astype(np.float64) @ b.astype(np.float64).T
    assert np.allclose(d, ref, rtol=1e-4, atol=1e-3 * np.sqrt(K)), np.abs(d - ref).max()
    if K > 16:
        # exchanging the two descriptor offsets reads the operands in a different order
        d2 = np.zeros_like(d)
        assert lib.orn_tc_selftest(K, N, int(bf16), mode | 1, a16.ctypes.data, b16.ctypes.data, d2.ctypes.data) == 0
        assert not np.allclose(d2, ref, rtol=1e-4, atol=1e-3 * np.sqrt(K))


def _small():
    scene = scenes.small_test_scene(96, 64)
    bvh = ornament.Bvh(scene)
    r = ornament.Renderer(bvh, device=0)
    r.set_resolution(96, 64)
    s = _lib.State()
    s.depth, s.inverted_gamma, s.iterations, s.ray_cast_epsilon = 8, 1.0, 1, 0.001
    r.set_state(s)
    r.set_camera(scene.camera.to_struct())
    return scene, bvh, r, s


def test_f64_render_matches_oracle_fp64_accumulation(oracle):
    scene, bvh, r, s = _small()
    mean = r.render_f64(6)
    cp = ol.make_params(scene.camera, 96, 64, depth=8, textures_count=bvh.scene_textures_count)
    acc64 = np.zeros((96 * 64, 4), np.float64)
    oracle.render(bvh, cp, 6, acc64=acc64)
    assert np.array_equal(mean[:, :3], acc64[:, :3] / acc64[:, 3:4])
    r.close()


def test_relmse_reduction_and_convergence():
    scene, bvh, r, s = _small()
    ref = r.render_f64(1024)
    errs = []
    for spp in (16, 64):
        r.set_resolution(96, 64)
        s.iterations = spp
        r.set_state(s)
        r.set_camera(scene.camera.to_struct())
        r.render()
        e, skipped = r.relmse(ref, return_skipped=True)
        acc = r.accumulation().astype(np.float64)
        x = acc[:, :3] / acc[:, 3:4]
        ok = np.isfinite(x).all(axis=1) & np.isfinite(ref[:, :3]).all(axis=1)
        assert skipped == int((~ok).sum())
        host = np.mean((x[ok] - ref[ok, :3]) ** 2 / (ref[ok, :3] ** 2 + 1e-2))
        assert abs(e - host) <= 1e-9 * max(host, 1e-12) + 1e-15
        errs.append(e)
    assert 2.0 < errs[0] / errs[1] < 8.0        # ~1/spp for an unbiased estimator
    r.close()
