"""Host-side checks that need no GPU: the C ABI library loads and exports
every function include/ornament_cuda.h declares, struct layouts, status
handling without a device, and the BVH builder's invariants (the rules of
src/bvh.zig)."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from zig_ornament_gb300 import _lib, ornament, scenes

ROOT = Path(__file__).resolve().parents[1]


def header_functions():
    text = (ROOT / "include" / "ornament_cuda.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(orn_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_function():
    lib = _lib.load()
    declared = header_functions()
    assert len(declared) >= 25
    for name in declared:
        assert hasattr(lib, name), name
    assert set(declared) == set(_lib.FUNCTIONS), set(declared) ^ set(_lib.FUNCTIONS)


def test_integration_bindings_call_declared_functions():
    """The Zig and C snippets a maintainer copies from INTEGRATION.md call
    only functions the header declares (and every declared function is
    named there or in the header's own documentation)."""
    text = (ROOT / "INTEGRATION.md").read_text()
    used = set(re.findall(r"\bc\.(orn_[a-z0-9_]+)\s*\(", text)) | set(re.findall(r"`(orn_[a-z0-9_]+)", text))
    declared = set(header_functions())
    header = (ROOT / "include" / "ornament_cuda.h").read_text()
    types = set(re.findall(r"\b(?:struct|enum)\s+(orn_[a-z0-9_]+)", header)) | {"orn_headless"}   # + the C driver
    # `orn_batch_*` style mentions name a family, not a function
    unknown = {u for u in used if u not in declared and u not in types and not u.endswith("_")}
    assert not unknown, unknown
    assert len(used & declared) >= 20


def test_struct_sizes_match_gpu_structs_zig():
    assert C.sizeof(_lib.BvhNode) == 64
    assert C.sizeof(_lib.Material) == 32
    assert C.sizeof(_lib.Camera) == 112
    assert C.sizeof(_lib.ConstantParams) == 144
    assert ornament.NODE_DTYPE.itemsize == 64 and ornament.MATERIAL_DTYPE.itemsize == 32


def test_status_strings_and_null_arguments():
    lib = _lib.load()
    assert lib.orn_status_string(0) == b"ok"
    assert lib.orn_status_string(6) == b"invalid scene data"
    out = C.c_void_p()
    assert lib.orn_create(None, 0, C.byref(out)) == 1
    assert lib.orn_render(None) == 1
    assert lib.orn_destroy(None) == 1
    assert lib.orn_bvh_build(None, C.byref(out)) == 1


def test_create_without_device_is_a_status(golden_bvh):
    lib = _lib.load()
    blob, keep = golden_bvh.blob()
    out = C.c_void_p()
    st = lib.orn_create(C.byref(blob), 0, C.byref(out))
    if st == 0:      # a GPU is present: this is not the case under test
        lib.orn_destroy(out)
        pytest.skip("a CUDA device is present")
    assert st == 5   # ORN_ERR_NO_DEVICE


def test_blob_validation_rejects_bad_indices_before_touching_a_device(golden_bvh):
    lib = _lib.load()
    bad = ornament.Bvh.from_arrays(**{k: getattr(golden_bvh, k) for k in
                                     ("tlas_nodes", "normals", "normal_indices", "uvs", "uv_indices",
                                      "transforms", "materials", "textures", "scene_textures_count")},
                                   blas_nodes=golden_bvh.blas_nodes.copy())
    bad.blas_nodes["left_or_custom_id"][-1] = 10 ** 6
    blob, keep = bad.blob()
    out = C.c_void_p()
    assert lib.orn_create(C.byref(blob), 0, C.byref(out)) == 6


# ---------------------------------------------------------------- builder


def check_invariants(scene, bvh):
    shapes = len(scene.spheres) + len(scene.meshes) + len(scene.mesh_instances)
    tris = [len(m.vertex_indices) // 3 for m in scene.meshes]
    # node counts (src/bvh.zig:17-21, 74-75)
    assert len(bvh.tlas_nodes) == 2 * shapes - 1
    assert len(bvh.blas_nodes) == sum(2 * t - 1 for t in tris)
    # children are appended before their parent (ids below the parent's)
    for arr in (bvh.tlas_nodes, bvh.blas_nodes):
        internal = np.nonzero(arr["node_type"] == 0)[0]
        assert (arr["left_or_custom_id"][internal] < internal).all()
        assert (arr["right_or_material_index"][internal] < internal).all()
    # TLAS: leaves are spheres/meshes, each with its own transform pair
    leaves = bvh.tlas_nodes[bvh.tlas_nodes["node_type"] != 0]
    assert len(leaves) == shapes
    assert sorted(leaves["transform_id"].tolist()) == list(range(shapes))
    assert len(bvh.transforms) == 2 * shapes
    assert (leaves["right_or_material_index"] < len(bvh.materials)).all()
    # BLAS: triangle leaves carry global triangle ids, each id once
    tri_nodes = bvh.blas_nodes[bvh.blas_nodes["node_type"] == 3]
    assert sorted(tri_nodes["left_or_custom_id"].tolist()) == list(range(sum(tris)))
    # the root of each mesh's BLAS is the last node of that mesh
    base = 0
    roots = set()
    for t in tris:
        base += 2 * t - 1
        roots.add(base - 1)
    mesh_leaves = leaves[leaves["node_type"] == 2]
    assert set(mesh_leaves["left_or_custom_id"].tolist()) <= roots
    # internal boxes contain their children's boxes
    for arr in (bvh.tlas_nodes,):
        for i in np.nonzero(arr["node_type"] == 0)[0][:200]:
            n = arr[i]
            for side, (mn_f, mx_f) in ((n["left_or_custom_id"], ("left_aabb_min_or_v0", "left_aabb_max_or_v1")),
                                       (n["right_or_material_index"], ("right_aabb_min_or_v2", "right_aabb_max_or_v3"))):
                c = arr[side]
                if c["node_type"] == 0:
                    cmin = np.minimum(c["left_aabb_min_or_v0"], c["right_aabb_min_or_v2"])
                    cmax = np.maximum(c["left_aabb_max_or_v1"], c["right_aabb_max_or_v3"])
                    assert (n[mn_f] <= cmin).all() and (n[mx_f] >= cmax).all()


@pytest.mark.parametrize("make", [lambda: scenes.small_test_scene(),
                                  lambda: scenes.spheres_scene(64, 36, reference_grid=True),
                                  lambda: scenes.instanced_meshes_scene(64, 36, n_blas=3, n_instances=20,
                                                                        tri_range=(500, 3000), texture_size=32)])
def test_builder_invariants(make):
    scene = make()
    check_invariants(scene, ornament.Bvh(scene))


def test_builder_is_deterministic_and_seeded():
    scene = scenes.instanced_meshes_scene(64, 36, n_blas=3, n_instances=20, tri_range=(500, 3000), texture_size=32)
    a, b = ornament.Bvh(scene), ornament.Bvh(scene)
    assert np.array_equal(a.tlas_nodes, b.tlas_nodes) and np.array_equal(a.blas_nodes, b.blas_nodes)
    c = ornament.Bvh(scene, seed=99)
    assert not np.array_equal(a.blas_nodes, c.blas_nodes)
    assert len(a.blas_nodes) == len(c.blas_nodes)


def test_builder_parallel_build_matches_small_meshes():
    """A mesh large enough for the threaded BLAS build gives the same tree as
    the same triangles split into the per-node order computed sequentially:
    checked through the invariants and a rebuild with a different thread
    schedule (two builds of the same big mesh are identical)."""
    scene = ornament.Scene()
    v, n, uv, idx = scenes.icosphere(130)   # 338k triangles -> threaded subtrees
    m = scene.createMesh(v, idx, n, idx, uv, idx, ornament.identity(), scene.lambertian((0.5, 0.5, 0.5, 1)))
    a, b = ornament.Bvh(scene), ornament.Bvh(scene)
    assert np.array_equal(a.blas_nodes, b.blas_nodes)
    check_invariants(scene, a)


def test_material_and_texture_indices_follow_first_use():
    """getMaterialIndex (src/bvh.zig:369-383): materials are numbered in TLAS
    leaf order; a textured material appends its texture then."""
    scene = scenes.small_test_scene()
    bvh = ornament.Bvh(scene)
    leaves = bvh.tlas_nodes[bvh.tlas_nodes["node_type"] != 0]
    order = leaves[np.argsort(leaves["transform_id"])]["right_or_material_index"]
    first_seen = []
    for m in order:
        if m not in first_seen:
            first_seen.append(m)
    assert first_seen == list(range(len(bvh.materials)))
    tex = bvh.materials["albedo_texture_index"]
    used = tex[tex != _lib.NO_TEXTURE]
    assert sorted(used.tolist()) == list(range(len(bvh.textures)))
    assert bvh.scene_textures_count == len(scene.textures)


def test_transforms_are_transposed_inverse_forward_pairs():
    scene = scenes.small_test_scene()
    bvh = ornament.Bvh(scene, row_major_transforms=True)
    col = ornament.Bvh(scene, row_major_transforms=False)
    for k in range(0, len(bvh.transforms), 2):
        inv = bvh.transforms[k].reshape(4, 4).T
        fwd = bvh.transforms[k + 1].reshape(4, 4).T
        assert np.allclose(inv @ fwd, np.eye(4), atol=1e-4)
        assert np.array_equal(col.transforms[k + 1].reshape(4, 4), fwd)


def test_empty_scene_and_empty_mesh_are_errors():
    with pytest.raises(_lib.OrnamentError) as e:
        ornament.Bvh(ornament.Scene())
    assert e.value.status == 2
    scene = ornament.Scene()
    scene.createMesh(np.zeros((0, 4)), np.zeros(0, np.uint32), np.zeros((0, 4)), np.zeros(0, np.uint32),
                     np.zeros((0, 2)), np.zeros(0, np.uint32), ornament.identity(), scene.lambertian((1, 1, 1, 1)))
    with pytest.raises(_lib.OrnamentError) as e:
        ornament.Bvh(scene)
    assert e.value.status == 2


# ---------------------------------------------------------------- scene API


def test_camera_matches_camera_zig_formulas():
    cam = ornament.Camera(ornament.f32x4(13, 2, 3, 1), ornament.f32x4(0, 0, 0, 1), ornament.f32x4(0, 1, 0, 0),
                          16 / 9, 20.0, 0.1, 10.0)
    w = np.array([13, 2, 3], np.float64) / np.linalg.norm([13, 2, 3])
    u = np.cross([0, 1, 0], w)
    u /= np.linalg.norm(u)
    v = np.cross(w, u)
    h = np.tan(np.radians(20.0) / 2)
    assert np.allclose(cam.horizontal[:3], 10 * 16 / 9 * 2 * h * u, atol=1e-5)
    assert np.allclose(cam.vertical[:3], 10 * 2 * h * v, atol=1e-5)
    assert np.allclose(cam.lower_left_corner[:3],
                       np.array([13, 2, 3]) - cam.horizontal[:3] / 2 - cam.vertical[:3] / 2 - 10 * w, atol=1e-4)
    assert cam.lens_radius == np.float32(0.05) and cam.dirty
    cam.dirty = False
    cam.setAspectRatio(1.0)
    assert cam.dirty and cam.getAspectRatio() == 1.0


def test_state_defaults_match_state_zig():
    s = ornament.State()
    assert (s.resolution.width, s.resolution.height, s.depth, s.flip_y, s.inverted_gamma, s.iterations,
            s.ray_cast_epsilon, s.current_iteration) == (500, 500, 10, False, 1.0, 1, 0.001, 0.0)
    s.setGamma(2.2)
    assert abs(s.getGamma() - 2.2) < 1e-6


def test_sphere_mesh_and_plane_mesh_shapes():
    scene = ornament.Scene()
    m = scene.createSphereMesh(ornament.f32x4(0, 1, 0, 1), 2.0, scene.dielectric(1.5))
    assert len(m.vertices) == 2 + 29 * 60
    assert len(m.vertex_indices) // 3 == 60 + 28 * 60 * 2 + 60
    assert np.allclose(m.aabb.min[:3], [-2, -1, -2], atol=1e-3) and np.allclose(m.aabb.max[:3], [2, 3, 2], atol=1e-3)
    p = scene.createPlaneMesh(ornament.f32x4(0, 5, 0, 1), 2.0, 3.0, ornament.f32x4(0, -1, 0, 0),
                              scene.diffuseLight((4, 4, 4, 1)))
    assert len(p.vertex_indices) == 6 and np.allclose(p.uvs, 0.5)
    assert np.allclose(p.aabb.min[:3], [-1, 5, -1.5], atol=1e-5)


def test_aabb_transform_is_exact_for_translation_and_scale():
    a = ornament.Aabb(ornament.f32x4(-1, -1, -1, 1), ornament.f32x4(1, 1, 1, 1))
    m = ornament.mul(ornament.scaling(2, 3, 4), ornament.translation(10, 0, -5))
    t = ornament.Aabb.transform(m, a)
    assert np.array_equal(t.min[:3], np.array([8, -3, -9], np.float32))
    assert np.array_equal(t.max[:3], np.array([12, 3, -1], np.float32))
