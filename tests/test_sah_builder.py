"""The SAH builder (ORN_BVH_SAH, a non-parity mode): a valid tree in the
reference's node format whose closest hits are the reference tree's, with
fewer node visits (CPU, through the oracle's Bvh::hit restatement)."""
import numpy as np

from zig_ornament_gb300 import ornament, scenes


def _rays(scene, w, h, n, seed):
    cam = scene.camera.to_struct()
    rs = np.random.default_rng(seed)
    px, py = rs.integers(0, w, n), rs.integers(0, h, n)
    u = ((px + rs.random(n)) / (w - 1)).astype(np.float32)[:, None]
    v = ((py + rs.random(n)) / (h - 1)).astype(np.float32)[:, None]
    o = np.array(cam.origin[:], np.float32)
    d = (np.array(cam.lower_left_corner[:], np.float32) + u * np.array(cam.horizontal[:], np.float32)
         + v * np.array(cam.vertical[:], np.float32) - o)
    prim = np.concatenate([np.broadcast_to(o, d.shape), d], 1)
    # and random rays from points inside the scene box
    o2 = rs.uniform(-60, 60, (n, 3)).astype(np.float32)
    d2 = rs.normal(size=(n, 3)).astype(np.float32)
    return np.concatenate([prim, np.concatenate([o2, d2], 1)]).astype(np.float32)


def test_sah_tree_shape_and_hits(oracle):
    scene = scenes.instanced_meshes_scene(160, 90, seed=3, n_blas=4, n_instances=60, tri_range=(2000, 9000),
                                          texture_size=64)
    ref = ornament.Bvh(scene)
    sah = ornament.Bvh(scene, builder="sah")
    assert len(sah.tlas_nodes) == len(ref.tlas_nodes) and len(sah.blas_nodes) == len(ref.blas_nodes)
    assert not np.array_equal(sah.blas_nodes.view(np.uint8), ref.blas_nodes.view(np.uint8))
    rays = _rays(scene, 160, 90, 20000, 5)
    h_ref, v_ref = oracle.trace_rays(ref, rays)
    h_sah, v_sah = oracle.trace_rays(sah, rays)
    assert np.array_equal(h_ref["hit"], h_sah["hit"])
    hit = h_ref["hit"] != 0
    assert hit.sum() > 5000
    same_t = h_ref["t"][hit] == h_sah["t"][hit]
    assert same_t.mean() > 0.999            # only equal-distance ties may differ
    # material (and texture) ids follow leaf creation order, so compare the
    # materials' values
    m_ref = ref.materials[h_ref["material_index"][hit][same_t]]
    m_sah = sah.materials[h_sah["material_index"][hit][same_t]]
    for f in ("albedo", "fuzz", "ior", "type"):
        assert np.array_equal(m_ref[f], m_sah[f]), f
    assert v_sah.mean() < 0.8 * v_ref.mean()


def test_sah_tree_with_spheres(oracle):
    scene = scenes.spheres_scene(80, 45, seed=0)
    ref = ornament.Bvh(scene)
    sah = ornament.Bvh(scene, builder="sah")
    rays = _rays(scene, 80, 45, 5000, 6)
    rays[5000:, :3] *= 0.2   # the sphere field is ~20 units wide
    h_ref, v_ref = oracle.trace_rays(ref, rays)
    h_sah, v_sah = oracle.trace_rays(sah, rays)
    assert np.array_equal(h_ref["hit"], h_sah["hit"])
    hit = h_ref["hit"] != 0
    assert (h_ref["t"][hit] == h_sah["t"][hit]).mean() > 0.999
    assert v_sah.mean() < v_ref.mean()
