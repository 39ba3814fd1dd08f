"""The plain-C headless frame loop (zig_ornament_gb300/driver/orn_headless.c)
over the C ABI: it builds, fails loudly without a device, and on a GPU its
framebuffer — sphere scene, JPEG planet texture, several frames, a camera
move that restarts accumulation — is bit-identical to the same frames
rendered through the Python binding, which the parity tests tie to the
oracle."""
import subprocess
from pathlib import Path

import numpy as np
import pytest

from zig_ornament_gb300 import _lib, build, ornament, textures

GOLDEN = Path(__file__).resolve().parent / "golden"
TEXTURE = GOLDEN / "jpeg" / "rgb444_128x96.jpg"
W, H, FRAMES, ITER, DEPTH, MOVE_AT = 96, 54, 4, 3, 8, 2


def _driver():
    build.build_library()
    return build.build_driver()


def _run(tmp_path):
    out = tmp_path / "run"
    res = subprocess.run([str(_driver()), "-w", str(W), "-h", str(H), "-frames", str(FRAMES),
                          "-iterations", str(ITER), "-depth", str(DEPTH), "-gamma", "2.2",
                          "-texture", str(TEXTURE), "-move-at", str(MOVE_AT), "-out", str(out)],
                         capture_output=True, text=True, timeout=300)
    return res, out


def test_driver_without_a_device_fails_loudly(tmp_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    res, _ = _run(tmp_path)
    assert res.returncode == 1
    assert "no CUDA device" in res.stderr


@pytest.mark.gpu
def test_driver_matches_the_python_binding(tmp_path):
    res, out = _run(tmp_path)
    assert res.returncode == 0, res.stderr
    assert res.stdout.count("frame ") == FRAMES
    fb = np.fromfile(f"{out}.fb", dtype=np.float32).reshape(W * H, 4)
    cams = np.fromfile(f"{out}.cam", dtype=np.uint8).reshape(-1, C_CAMERA_SIZE)
    assert len(cams) == 2

    scene = ornament.Scene()
    ground = scene.lambertian((0.5, 0.5, 0.5, 1.0))
    glass = scene.dielectric(1.5)
    planet = scene.lambertian(textures.load_texture(scene, TEXTURE, device=0))
    metal = scene.metal((0.7, 0.6, 0.5, 1.0), 0.0)
    scene.attachSphere(scene.createSphere((0.0, -1000.0, 0.0, 1.0), 1000.0, ground))
    scene.attachSphere(scene.createSphere((0.0, 1.0, 0.0, 1.0), 1.0, glass))
    scene.attachSphere(scene.createSphere((-4.0, 1.0, 0.0, 1.0), 1.0, planet))
    scene.attachSphere(scene.createSphere((4.0, 1.0, 0.0, 1.0), 1.0, metal))
    bvh = ornament.Bvh(scene)
    r = ornament.Renderer(bvh, device=0)
    r.set_resolution(W, H)
    st = r.get_state()    # the library's defaults, as the driver starts from them
    st.depth, st.iterations = DEPTH, ITER
    st.inverted_gamma = float(np.float32(1.0) / np.float32(2.2))
    r.set_state(st)
    r.set_camera(_lib.Camera.from_buffer_copy(cams[0].tobytes()))
    for f in range(FRAMES):
        if f == MOVE_AT:
            r.set_camera(_lib.Camera.from_buffer_copy(cams[1].tobytes()))
        r.render()
    ours = r.framebuffer()
    r.close()
    assert np.array_equal(ours.view(np.uint32), fb.view(np.uint32))
    assert np.isfinite(fb).all() and fb[:, :3].max() > 0.05


C_CAMERA_SIZE = 112
