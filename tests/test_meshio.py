"""OBJ loading (meshio.read_obj / load_mesh): triangulation, joined
vertices, generated normals, normalisation, and a render of a loaded mesh
through the oracle (CPU)."""
import numpy as np
import pytest

from zig_ornament_gb300 import meshio, ornament

CUBE = """# unit cube, quads, no normals or uvs
v 0 0 0
v 1 0 0
v 1 1 0
v 0 1 0
v 0 0 1
v 1 0 1
v 1 1 1
v 0 1 1
f 1 4 3 2
f 5 6 7 8
f 1 2 6 5
f 2 3 7 6
f 3 4 8 7
f 4 1 5 8
"""

QUAD_UV_N = """v -1 -1 0
v 1 -1 0
v 1 1 0
v -1 1 0
vt 0 0
vt 1 0
vt 1 1
vt 0 1
vn 0 0 2
f 1/1/1 2/2/1 3/3/1
f -4/-4/-1 -2/-2/-1 -1/-1/-1
"""


def _write(tmp_path, text, name="m.obj"):
    p = tmp_path / name
    p.write_text(text)
    return p


def test_cube_triangulated_with_smooth_normals(tmp_path):
    m = meshio.read_obj(_write(tmp_path, CUBE))
    assert len(m.indices) == 36 and len(m.vertices) == 8      # 12 triangles, corners joined per position
    assert m.uvs.shape == (0, 2)
    n = m.normals[:, :3]
    assert np.allclose(np.linalg.norm(n, axis=1), 1.0, atol=1e-6)
    # a cube corner's smooth normal points out along the diagonal
    c = m.vertices[:, :3] - 0.5
    assert np.all(np.sum(n * c, axis=1) > 0)


def test_quad_with_uvs_normals_and_negative_indices(tmp_path):
    m = meshio.read_obj(_write(tmp_path, QUAD_UV_N))
    assert len(m.indices) == 6 and len(m.vertices) == 4
    assert np.allclose(m.normals[:, :3], [0, 0, 1])
    # each vertex keeps its own uv
    for i in range(4):
        p = m.vertices[i, :2]
        assert np.allclose(m.uvs[i], (p + 1) / 2)


def test_distinct_corners_are_not_joined(tmp_path):
    text = "v 0 0 0\nv 1 0 0\nv 0 1 0\nvt 0 0\nvt 1 1\nf 1/1 2/1 3/1\nf 1/2 3/2 2/2\n"
    m = meshio.read_obj(_write(tmp_path, text))
    assert len(m.vertices) == 6


def test_errors(tmp_path):
    with pytest.raises(ValueError):
        meshio.read_obj(_write(tmp_path, "v 0 0 0\nf 1 2 3\n"))
    with pytest.raises(ValueError):
        meshio.read_obj(_write(tmp_path, "v 0 0 0\n"))
    with pytest.raises(ValueError):
        meshio.read_obj(_write(tmp_path, "v 0 0 0\nv 1 0 0\nf 1 2\n"))


def test_load_mesh_normalises_and_renders(tmp_path, oracle):
    from oracle import oracle_lib as ol
    scene = ornament.Scene()
    mat = scene.lambertian((0.7, 0.3, 0.2, 1.0))
    mesh = meshio.load_mesh(scene, _write(tmp_path, CUBE), ornament.identity(), mat)
    v = mesh.vertices[:, :3]
    assert np.allclose(v.min(axis=0), -0.5) and np.allclose(v.max(axis=0), 0.5)
    scene.attachMesh(mesh)
    scene.camera = ornament.Camera(ornament.f32x4(2, 1.5, 3, 1), ornament.f32x4(0, 0, 0, 1),
                                   ornament.f32x4(0, 1, 0, 0), 1.5, 40.0, 0.0, 3.0)
    bvh = ornament.Bvh(scene)
    assert len(bvh.blas_nodes) == 2 * 12 - 1
    cp = ol.make_params(scene.camera, 48, 32, depth=4)
    acc, _, _, _ = oracle.render(bvh, cp, 2)
    mean = acc[:, :3] / acc[:, 3:]
    assert np.isfinite(mean).all()
    # the cube covers the image centre: its pixels are darker than the sky
    centre = mean.reshape(32, 48, 3)[14:18, 22:26].mean()
    corner = mean.reshape(32, 48, 3)[0:3, 0:3].mean()
    assert centre < corner
