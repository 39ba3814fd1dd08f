"""The JPEG texture loader on the GPU: decoded pixels against the float64
oracle (oracle/jpeg.py) within one level (FP32 rounding), against NVIDIA's
nvJPEG (an independent decoder, when the library is present), and a texture
loaded this way rendered bit-exact against the CPU oracle."""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest

from oracle import jpeg as oj
from oracle import oracle_lib as ol
from zig_ornament_gb300 import _lib, ornament, scenes, textures

from test_gpu_parity import bits, make_state

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden"
FIX = np.load(GOLDEN / "jpeg_fixtures.npz")
NAMES = sorted({k.split("/")[0] for k in FIX.files})


def _data(name):
    return (GOLDEN / "jpeg" / f"{name}.jpg").read_bytes()


@pytest.mark.parametrize("flip", [True, False], ids=["flip", "noflip"])
@pytest.mark.parametrize("name", NAMES)
def test_pixels_match_the_oracle(name, flip):
    got = textures.read_jpeg(_data(name), flip_y=flip, device=0)
    want = oj.decode_fixture(FIX, name, flip_y=flip)
    diff = np.abs(got.astype(int) - want.astype(int))
    assert diff.max() <= 1, (name, diff.max())
    assert (diff == 0).mean() > 0.99
    assert (got[..., 3] == 255).all()


def _nvjpeg():
    for cand in ("libnvjpeg.so.13", "libnvjpeg.so", "/usr/local/cuda/lib64/libnvjpeg.so"):
        try:
            return C.CDLL(cand)
        except OSError:
            continue
    return None


class _NvImage(C.Structure):
    _fields_ = [("channel", C.c_void_p * 4), ("pitch", C.c_size_t * 4)]


def _nvjpeg_rgb(lib, data, w, h):
    import torch
    handle, state = C.c_void_p(), C.c_void_p()
    assert lib.nvjpegCreateSimple(C.byref(handle)) == 0
    assert lib.nvjpegJpegStateCreate(handle, C.byref(state)) == 0
    try:
        buf = torch.zeros(h * w * 3, dtype=torch.uint8, device="cuda")
        img = _NvImage()
        img.channel[0] = buf.data_ptr()
        img.pitch[0] = w * 3
        torch.cuda.synchronize()
        st = lib.nvjpegDecode(handle, state, C.c_char_p(data), C.c_size_t(len(data)), 5, C.byref(img),
                              C.c_void_p(0))   # NVJPEG_OUTPUT_RGBI on the legacy default stream
        torch.cuda.synchronize()
        assert st == 0, f"nvjpegDecode status {st}"
        return buf.cpu().numpy().reshape(h, w, 3)
    finally:
        lib.nvjpegJpegStateDestroy(state)
        lib.nvjpegDestroy(handle)


@pytest.mark.parametrize("name", [n for n in NAMES if n != "rgb_adobe"])
def test_pixels_match_nvjpeg(name):
    lib = _nvjpeg()
    if lib is None:
        pytest.skip("nvJPEG is not installed")
    w, h, n = (int(v) for v in FIX[f"{name}/size"])
    ref = _nvjpeg_rgb(lib, _data(name), w, h).astype(int)
    got = textures.read_jpeg(_data(name), flip_y=False, device=0)[..., :3].astype(int)
    diff = np.abs(got - ref)
    subsampled = any(tuple(s) != (1, 1) for s in FIX[f"{name}/sampling"]) and n == 3
    print(f"{name}: max |ours - nvJPEG| = {diff.max()}, mean {diff.mean():.3f}")
    if subsampled:   # chroma filters may differ (replication here)
        assert diff.mean() < 4.0
    else:
        assert diff.max() <= 4 and diff.mean() < 0.5


def test_loaded_texture_renders_like_the_oracle(oracle):
    scene = scenes.spheres_scene(64, 36, seed=0)
    tex = textures.load_texture(scene, GOLDEN / "jpeg" / "rgb444_128x96.jpg", device=0)
    assert tex.width == 128 and tex.height == 96
    scene.attachSphere(scene.createSphere((0.0, 1.0, 0.0, 1.0), 1.0, scene.lambertian(tex)))
    bvh = ornament.Bvh(scene)
    r = ornament.Renderer(bvh, device=0)
    r.set_resolution(64, 36)
    r.set_state(make_state(depth=6, gamma=1.0, iterations=2))
    r.set_camera(scene.camera.to_struct())
    r.render()
    acc, rng, _ = r.progress()
    cp = ol.make_params(scene.camera, 64, 36, depth=6, textures_count=bvh.scene_textures_count)
    oacc, orng, _, _ = oracle.render(bvh, cp, 2)
    assert np.array_equal(rng, orng)
    assert np.array_equal(bits(acc), bits(oacc))
    r.close()
