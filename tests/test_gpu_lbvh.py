"""The GPU BLAS builder (ORN_BVH_LBVH, a non-parity mode): linear BVHs built
on the device.  The tree must be valid in the reference's node format, give
the reference tree's closest hits (through the oracle's traversal) and render
bit for bit like the oracle on that same tree; builds are deterministic."""
import time

import numpy as np
import pytest

from oracle import oracle_lib as ol
from zig_ornament_gb300 import _lib, ornament, scenes

from test_abi_and_builder import check_invariants
from test_gpu_parity import KERNELS, KERNEL_IDS, bits, make_state
from test_sah_builder import _rays


def _blas_boxes_contain_children(bvh):
    arr = bvh.blas_nodes
    tri = arr["node_type"] == 3
    lo = np.where(tri[:, None], np.minimum(np.minimum(arr["left_aabb_min_or_v0"], arr["left_aabb_max_or_v1"]),
                                           arr["right_aabb_min_or_v2"]),
                  np.minimum(arr["left_aabb_min_or_v0"], arr["right_aabb_min_or_v2"]))
    hi = np.where(tri[:, None], np.maximum(np.maximum(arr["left_aabb_min_or_v0"], arr["left_aabb_max_or_v1"]),
                                           arr["right_aabb_min_or_v2"]),
                  np.maximum(arr["left_aabb_max_or_v1"], arr["right_aabb_max_or_v3"]))
    internal = np.nonzero(~tri)[0]
    l = arr["left_or_custom_id"][internal]
    r = arr["right_or_material_index"][internal]
    # the stored child boxes are exactly the children's bounds
    assert np.array_equal(arr["left_aabb_min_or_v0"][internal], lo[l])
    assert np.array_equal(arr["left_aabb_max_or_v1"][internal], hi[l])
    assert np.array_equal(arr["right_aabb_min_or_v2"][internal], lo[r])
    assert np.array_equal(arr["right_aabb_max_or_v3"][internal], hi[r])
    # every node but the per-mesh roots is referenced exactly once
    refs = np.bincount(np.concatenate([l, r]), minlength=len(arr))
    assert refs.max() == 1


def _scene():
    return scenes.instanced_meshes_scene(160, 90, seed=3, n_blas=4, n_instances=60, tri_range=(2000, 9000),
                                         texture_size=64)


@pytest.mark.gpu
def test_lbvh_tree_is_valid_and_deterministic():
    scene = _scene()
    a = ornament.Bvh(scene, builder="lbvh")
    b = ornament.Bvh(scene, builder="lbvh")
    check_invariants(scene, a)
    _blas_boxes_contain_children(a)
    assert np.array_equal(a.blas_nodes.view(np.uint8), b.blas_nodes.view(np.uint8))
    assert np.array_equal(a.tlas_nodes.view(np.uint8), b.tlas_nodes.view(np.uint8))
    # the TLAS is the SAH builder's
    s = ornament.Bvh(scene, builder="sah")
    assert np.array_equal(a.tlas_nodes.view(np.uint8), s.tlas_nodes.view(np.uint8))


@pytest.mark.gpu
def test_lbvh_single_and_two_triangle_meshes():
    scene = ornament.Scene()
    mat = scene.lambertian((0.5, 0.5, 0.5, 1))
    for nt in (1, 2, 3):
        v = np.zeros((3 * nt, 4), np.float32)
        v[:, 3] = 1
        for k in range(nt):
            v[3 * k:3 * k + 3, :3] = [[k, 0, 0], [k + 1, 0, 0], [k, 1, 0.5 * k]]
        idx = np.arange(3 * nt, dtype=np.uint32)
        nrm = np.tile(np.array([[0, 0, 1, 0]], np.float32), (3 * nt, 1))
        uv = np.zeros((3 * nt, 2), np.float32)
        scene.createMesh(v, idx, nrm, idx, uv, idx, ornament.identity(), mat)
    bvh = ornament.Bvh(scene, builder="lbvh")
    check_invariants(scene, bvh)
    _blas_boxes_contain_children(bvh)


@pytest.mark.gpu
def test_lbvh_hits_match_the_reference_tree(oracle):
    scene = _scene()
    ref = ornament.Bvh(scene)
    lb = ornament.Bvh(scene, builder="lbvh")
    rays = _rays(scene, 160, 90, 20000, 5)
    h_ref, v_ref = oracle.trace_rays(ref, rays)
    h_lb, v_lb = oracle.trace_rays(lb, rays)
    assert np.array_equal(h_ref["hit"], h_lb["hit"])
    hit = h_ref["hit"] != 0
    assert hit.sum() > 5000
    same_t = h_ref["t"][hit] == h_lb["t"][hit]
    assert same_t.mean() > 0.999            # only equal-distance ties may differ
    m_ref = ref.materials[h_ref["material_index"][hit][same_t]]
    m_lb = lb.materials[h_lb["material_index"][hit][same_t]]
    for f in ("albedo", "fuzz", "ior", "type"):
        assert np.array_equal(m_ref[f], m_lb[f]), f
    print(f"mean visits per ray: reference tree {v_ref.mean():.1f}, LBVH {v_lb.mean():.1f}")
    assert v_lb.mean() < v_ref.mean()


@pytest.mark.gpu
@pytest.mark.parametrize("kernel", KERNELS, ids=KERNEL_IDS)
def test_lbvh_tree_renders_like_the_oracle(oracle, kernel):
    scene = scenes.instanced_meshes_scene(96, 54, seed=1, n_blas=4, n_instances=40, tri_range=(2000, 8000),
                                          texture_size=128)
    bvh = ornament.Bvh(scene, builder="lbvh")
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


@pytest.mark.gpu
def test_lbvh_builds_a_large_mesh_faster_than_the_cpu_builders():
    scene = ornament.Scene()
    v, n, uv, idx = scenes.icosphere(200)   # 800k triangles
    scene.createMesh(v, idx, n, idx, uv, idx, ornament.identity(), scene.lambertian((0.5, 0.5, 0.5, 1)))
    ornament.Bvh(scene, builder="lbvh")     # device and CUB warm-up
    times = {}
    for b in ("reference", "sah", "lbvh"):
        t0 = time.perf_counter()
        bvh = ornament.Bvh(scene, builder=b)
        times[b] = time.perf_counter() - t0
    check_invariants(scene, bvh)
    _blas_boxes_contain_children(bvh)
    print("build seconds:", {k: round(t, 3) for k, t in times.items()})
    assert times["lbvh"] < times["sah"]


def test_lbvh_without_a_device_fails_loudly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    with pytest.raises(_lib.OrnamentError, match="NO_DEVICE"):
        ornament.Bvh(scenes.small_test_scene(), builder="lbvh")
