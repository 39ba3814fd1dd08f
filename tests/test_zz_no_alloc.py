"""orn_render_noalloc — rendering for callers that cannot allocate device
memory while they render (a frame loop that must never call cudaMalloc, or a
host that hands the renderer a fixed memory budget).  The entry point works
in a fixed array inside the library and writes into device buffers the
caller owns.

Checked through the C ABI against the existing entry point, orn_render on the
same context: two calls in a row (a 3-pass render, then a 2-pass
continuation) give the same accumulation, RNG states and framebuffer, bit for
bit — the tolerance of every parity test here.  This file is collected last
so that a run stopping at the first failure has run every other test; it
also passes alone in a fresh process (the first call does the per-device
set-up)."""
import ctypes as C

import numpy as np
import pytest

from zig_ornament_gb300 import _lib, ornament, scenes

pytestmark = pytest.mark.gpu

W, H = 96, 64


def state(iterations):
    s = _lib.State()
    s.depth, s.flip_y, s.iterations, s.ray_cast_epsilon = 8, 1, iterations, 0.001
    s.inverted_gamma = float(np.float32(1.0) / np.float32(2.2))
    s.semantics, s.kernel, s.spp_per_launch = _lib.SEMANTICS_HIP, _lib.KERNEL_MEGA, 0
    return s


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def test_noalloc_matches_render_on_two_calls():
    import torch
    lib = _lib.load()
    scene = scenes.small_test_scene(W, H)
    bvh = ornament.Bvh(scene)
    r = ornament.Renderer(bvh, device=0)
    r.set_resolution(W, H)
    r.set_state(state(3))
    r.set_camera(scene.camera.to_struct())
    cp = r.peek_constant_params()            # first pass: current_iteration = 1
    assert cp.current_iteration == 1.0

    # caller-owned device buffers, a fresh target: RNG seeded with the pixel index
    dev = torch.device("cuda", 0)
    acc = torch.zeros((W * H, 4), dtype=torch.float32, device=dev)
    rng = torch.arange(W * H, dtype=torch.int32, device=dev)
    fb = torch.zeros((W * H, 4), dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream

    def noalloc(params, spp):
        st = lib.orn_render_noalloc(r.handle, C.byref(params), spp, acc.data_ptr(), rng.data_ptr(),
                                    fb.data_ptr(), stream)
        assert st == 0, lib.orn_status_string(st)
        torch.cuda.synchronize(dev)
        return acc.cpu().numpy().copy(), rng.cpu().numpy().view(np.uint32).copy(), fb.cpu().numpy().copy()

    a1, g1, f1 = noalloc(cp, 3)
    cp2 = _lib.ConstantParams.from_buffer_copy(bytes(cp))
    cp2.current_iteration = 4.0
    a2, g2, f2 = noalloc(cp2, 2)

    # the existing entry point, same context and state
    r.render()
    ra1, rg1, ci1 = r.progress()
    rf1 = r.framebuffer().copy()
    r.set_state(state(2))
    r.render()
    ra2, rg2, ci2 = r.progress()
    rf2 = r.framebuffer().copy()
    assert (ci1, ci2) == (3.0, 5.0)

    for got, want in ((a1, ra1), (g1, rg1), (f1, rf1), (a2, ra2), (g2, rg2), (f2, rf2)):
        assert np.array_equal(bits(got), bits(want))
    assert (a2[:, 3] == 5.0).all()
    r.synchronize()                          # no device-side error was recorded


def test_noalloc_rejects_oversized_frames():
    lib = _lib.load()
    scene = scenes.small_test_scene(W, H)
    r = ornament.Renderer(ornament.Bvh(scene), device=0)
    r.set_resolution(W, H)
    r.set_state(state(1))
    r.set_camera(scene.camera.to_struct())
    cp = r.peek_constant_params()
    cp.width, cp.height = 1024, 1024          # 1 Mi pixels > ORN_NOALLOC_MAX_PIXELS
    assert 1024 * 1024 > _lib.NOALLOC_MAX_PIXELS
    st = lib.orn_render_noalloc(r.handle, C.byref(cp), 1, 16, 16, 16, None)
    assert st == 1                            # ORN_ERR_INVALID_ARGUMENT, nothing launched
    cp = r.peek_constant_params()
    cp.depth = _lib.NOALLOC_MAX_DEPTH + 1     # the call would queue spp * (depth + 1) + 2 launch pairs
    st = lib.orn_render_noalloc(r.handle, C.byref(cp), 1, 16, 16, 16, None)
    assert st == 1
    r.close()


def test_noalloc_keeps_the_callers_device():
    import torch
    lib = _lib.load()
    scene = scenes.small_test_scene(W, H)
    r = ornament.Renderer(ornament.Bvh(scene), device=0)
    r.set_resolution(W, H)
    r.set_state(state(1))
    r.set_camera(scene.camera.to_struct())
    cp = r.peek_constant_params()
    dev = torch.device("cuda", 0)
    acc = torch.zeros((W * H, 4), dtype=torch.float32, device=dev)
    rng = torch.arange(W * H, dtype=torch.int32, device=dev)
    fb = torch.zeros((W * H, 4), dtype=torch.float32, device=dev)
    before = torch.cuda.current_device()
    for _ in range(3):   # later calls also read the previous call's error report
        st = lib.orn_render_noalloc(r.handle, C.byref(cp), 1, acc.data_ptr(), rng.data_ptr(), fb.data_ptr(),
                                    torch.cuda.current_stream(dev).cuda_stream)
        assert st == 0, lib.orn_status_string(st)
        torch.cuda.synchronize(dev)
    assert torch.cuda.current_device() == before
    r.synchronize()
    r.close()
