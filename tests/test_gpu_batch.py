"""Batched rendering (orn_batch_*): one persistent launch over many contexts
equals each context's own orn_render bit for bit; the frame is replayed as
a CUDA graph across frames and launch shapes; the autotuner leaves the
contexts untouched and round-trips its JSON cache."""
import json

import numpy as np
import pytest

from zig_ornament_gb300 import _lib, ornament, scenes

pytestmark = pytest.mark.gpu


def _views():
    """(scene, width, height, iterations, flip_y, gamma) of uneven contexts."""
    out = []
    out.append((scenes.small_test_scene(96, 64), 96, 64, 3, False, 1.0))
    out.append((scenes.spheres_scene(160, 90, seed=0), 160, 90, 5, True, 2.2))
    out.append((scenes.cornell_box_scene(64, 48), 64, 48, 2, False, 1.0))
    for k, (sc, w, h, spp) in enumerate(scenes.batch_scenes(count=3, seed=7, tri_range=(1_000, 20_000),
                                                            instance_range=(1, 64), spp_range=(1, 4),
                                                            resolutions=((48, 32), (80, 45), (33, 17)),
                                                            texture_size=64)):
        out.append((sc, w, h, spp, k == 1, 1.0))
    return out


def _context(view, semantics=0):
    sc, w, h, spp, flip, gamma = view
    bvh = ornament.Bvh(sc, row_major_transforms=True)
    r = ornament.Renderer(bvh, 0)
    r.set_resolution(w, h)
    st = ornament.State()
    st.depth = 6
    st.iterations = spp
    st.setFlipY(flip)
    st.setGamma(gamma)
    st.semantics = semantics
    r.set_state(st.to_struct())
    r.set_camera(sc.camera.to_struct())
    return r


def _images(r):
    r.synchronize()
    return r.accumulation().copy(), r.framebuffer().copy(), r.progress()


@pytest.mark.parametrize("semantics", [0, 1])
def test_batch_equals_individual_renders(semantics):
    views = _views()
    solo = [_context(v, semantics) for v in views]
    batched = [_context(v, semantics) for v in views]
    batch = ornament.Batch(batched)
    for frame in range(2):
        for r in solo:
            r.render()
        batch.render()
        for i, (a, b) in enumerate(zip(solo, batched)):
            acc_a, fb_a, prog_a = _images(a)
            acc_b, fb_b, prog_b = _images(b)
            assert np.array_equal(acc_a.view(np.uint32), acc_b.view(np.uint32)), (frame, i)
            assert np.array_equal(fb_a.view(np.uint32), fb_b.view(np.uint32)), (frame, i)
            assert np.array_equal(prog_a[1], prog_b[1]), (frame, i)   # RNG states
            assert prog_a[2] == prog_b[2]                               # current_iteration
    batch.synchronize()
    assert batch.last_render_ms() > 0
    batch.close()
    for r in solo + batched:
        r.close()


def test_batch_launch_shapes_agree_and_camera_restart():
    views = _views()[:4]
    ref = [_context(v) for v in views]
    for r in ref:
        r.render()
    imgs = [_images(r)[0] for r in ref]
    for cfg in ({"block": 64, "blocks_per_sm": 4, "shade_threshold": 4},
                {"block": 192, "blocks_per_sm": 2, "shade_threshold": 16},
                {"block": 128, "blocks_per_sm": 6, "shade_threshold": 8}):
        ctxs = [_context(v) for v in views]
        b = ornament.Batch(ctxs)
        b.set_config(**cfg)
        b.render()
        for img, r in zip(imgs, ctxs):
            assert np.array_equal(img.view(np.uint32), _images(r)[0].view(np.uint32)), cfg
        # a camera change restarts that context's accumulation, as in orn_render
        ctxs[0].set_camera(views[0][0].camera.to_struct())
        b.render()
        assert np.array_equal(imgs[0][:, 3], _images(ctxs[0])[0][:, 3])
        b.close()
        for r in ctxs:
            r.close()
    with pytest.raises(_lib.OrnamentError):
        b = ornament.Batch([_context(views[0])])
        b.set_config(block=96)


def test_batch_tuner_cache(tmp_path):
    views = _views()
    ctxs = [_context(v) for v in views]
    b = ornament.Batch(ctxs)
    path = tmp_path / "tune.json"
    chosen = b.tune(path)
    assert chosen["tuned"] and chosen["block"] in (64, 128, 192)
    data = json.loads(path.read_text())
    assert len(data) == 1
    entry = next(iter(data.values()))
    assert entry["block"] == chosen["block"] and entry["blocks_per_sm"] == chosen["blocks_per_sm"]
    assert entry["ms"] > 0
    # tuning did not touch the contexts: a render now equals a fresh context's
    b.render()
    for v, r in zip(views, ctxs):
        fresh = _context(v)
        fresh.render()
        assert np.array_equal(_images(fresh)[0].view(np.uint32), _images(r)[0].view(np.uint32))
        fresh.close()
    # a second batch of the same workload reads the choice back from the file
    ctxs2 = [_context(v) for v in views]
    b2 = ornament.Batch(ctxs2)
    again = b2.tune(path)
    assert again == chosen
    b.close()
    b2.close()
    for r in ctxs + ctxs2:
        r.close()


def test_batch_rejects_mixed_semantics():
    views = _views()[:2]
    a = _context(views[0], 0)
    c = _context(views[1], 1)
    b = ornament.Batch([a, c])
    with pytest.raises(_lib.OrnamentError):
        b.render()
    b.close()
    a.close()
    c.close()
