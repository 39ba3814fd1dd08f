"""GPU: the persistent wavefront's launch parameters (orn_wave_set_config)
and their autotuner (orn_wave_tune).  Every block shape, fetch threshold
and round length renders the megakernel's bits; the tuner works on scratch
targets, leaves the context's image untouched and reads its choice back
from its cache file."""
import json

import numpy as np
import pytest

from zig_ornament_gb300 import _lib, ornament, scenes

pytestmark = pytest.mark.gpu

W, H = 320, 180


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def _renderer(bvh, scene, kernel, iterations=3):
    r = ornament.Renderer(bvh, device=0)
    r.set_resolution(W, H)
    s = _lib.State()
    s.depth, s.inverted_gamma, s.iterations, s.ray_cast_epsilon = 8, 1.0, iterations, 0.001
    s.kernel = kernel
    r.set_state(s)
    r.set_camera(scene.camera.to_struct())
    return r


@pytest.fixture(scope="module")
def instanced():
    scene = scenes.instanced_meshes_scene()
    return scene, ornament.Bvh(scene)


@pytest.fixture(scope="module")
def mega_progress(instanced):
    scene, bvh = instanced
    r = _renderer(bvh, scene, _lib.KERNEL_MEGA)
    r.render()
    out = r.progress()
    fb = r.framebuffer().copy()
    r.close()
    return out, fb


@pytest.mark.parametrize("shape", [0, 1, 2, 3])
@pytest.mark.parametrize("fetch,steps", [(1, 32), (4, 64), (32, 32)])
def test_every_configuration_renders_the_megakernels_bits(instanced, mega_progress, shape, fetch, steps):
    scene, bvh = instanced
    r = _renderer(bvh, scene, _lib.KERNEL_WAVEFRONT)
    r.set_wave_config(shape=shape, fetch=fetch, steps=steps)
    assert r.wave_config() == {"shape": shape, "fetch": fetch, "steps": steps, "tuned": False}
    r.render()
    (acc, rng, ci), fb = r.progress(), r.framebuffer()
    (macc, mrng, mci), mfb = mega_progress
    assert np.array_equal(bits(acc), bits(macc)) and np.array_equal(rng, mrng) and ci == mci
    assert np.array_equal(bits(fb), bits(mfb))
    r.close()


def test_invalid_configurations_are_rejected(instanced):
    scene, bvh = instanced
    r = _renderer(bvh, scene, _lib.KERNEL_WAVEFRONT)
    for bad in [dict(shape=4), dict(fetch=0), dict(fetch=33), dict(steps=16), dict(steps=48), dict(steps=128)]:
        with pytest.raises(_lib.OrnamentError):
            r.set_wave_config(**bad)
    assert r.wave_config() == {"shape": 0, "fetch": 4, "steps": 32, "tuned": False}
    r.close()


def test_tuner_keeps_the_image_and_caches_its_choice(instanced, mega_progress, tmp_path):
    scene, bvh = instanced
    path = tmp_path / "wave.json"
    r = _renderer(bvh, scene, _lib.KERNEL_WAVEFRONT)
    chosen = r.wave_tune(path)
    assert chosen["tuned"] and 0 <= chosen["shape"] < 4
    assert chosen["fetch"] in (2, 4, 8) and chosen["steps"] in (32, 64)
    data = json.loads(path.read_text())
    assert len(data) == 1
    entry = next(iter(data.values()))
    assert {k: entry[k] for k in ("shape", "fetch", "steps")} == {k: chosen[k] for k in ("shape", "fetch", "steps")}
    assert entry["ms"] > 0
    # tuning rendered into scratch targets: the first render still starts
    # from the context's own (fresh) state and equals the megakernel's
    r.render()
    (acc, rng, _), (macc, mrng, _) = r.progress(), mega_progress[0]
    assert np.array_equal(bits(acc), bits(macc)) and np.array_equal(rng, mrng)
    r.close()
    # a second context of the same workload reads the choice back
    r2 = _renderer(bvh, scene, _lib.KERNEL_WAVEFRONT)
    assert r2.wave_tune(path) == chosen
    r2.close()
