"""The watertight triangle test (orn_state.triangle_test = WATERTIGHT, a
non-parity option): rays from inside a closed mesh through its vertices and
edges all hit, and away from edges it agrees with the reference's test."""
import numpy as np
import pytest

from zig_ornament_gb300 import _lib, ornament, scenes

pytestmark = pytest.mark.gpu


def _closed_mesh_renderer(test):
    scene = ornament.Scene()
    v, n, uv, idx = scenes.icosphere(24)
    m = scene.createMesh(v, idx, n, idx, uv, idx, ornament.identity(), scene.lambertian((0.5, 0.5, 0.5, 1.0)))
    scene.attachMesh(m)
    scene.camera = ornament.Camera(ornament.f32x4(0, 0, 5, 1), ornament.f32x4(0, 0, 0, 1),
                                   ornament.f32x4(0, 1, 0, 0), 1.0, 40.0, 0.0, 5.0)
    r = ornament.Renderer(ornament.Bvh(scene), device=0)
    st = ornament.State()
    st.triangle_test = test
    r.set_state(st.to_struct())
    return r, v[:, :3].astype(np.float32), idx.reshape(-1, 3)


def _edge_rays(v, tris):
    """From the centre through every vertex and every edge midpoint."""
    e = np.concatenate([tris[:, [0, 1]], tris[:, [1, 2]], tris[:, [2, 0]]])
    mids = 0.5 * (v[e[:, 0]] + v[e[:, 1]])
    d = np.concatenate([v, mids]).astype(np.float32)
    return np.concatenate([np.zeros_like(d), d], 1).astype(np.float32)


def test_watertight_closed_mesh_has_no_cracks():
    r_w, v, tris = _closed_mesh_renderer(_lib.TRIANGLE_WATERTIGHT)
    r_m, _, _ = _closed_mesh_renderer(_lib.TRIANGLE_MOLLER_TRUMBORE)
    rays = _edge_rays(v, tris)
    hw, _ = r_w.trace_rays(rays)
    hm, _ = r_m.trace_rays(rays)
    miss_w = int((hw["hit"] == 0).sum())
    miss_m = int((hm["hit"] == 0).sum())
    print(f"{len(rays)} rays through vertices and edge midpoints: misses watertight {miss_w}, "
          f"Moller-Trumbore {miss_m}")
    assert miss_w == 0
    # every hit lies on the unit sphere's polyhedron: 0.99 < t < 1.0001
    assert np.all(hw["t"] > 0.98) and np.all(hw["t"] < 1.0001)
    r_w.close()
    r_m.close()


def test_watertight_agrees_away_from_edges():
    r_w, v, tris = _closed_mesh_renderer(_lib.TRIANGLE_WATERTIGHT)
    r_m, _, _ = _closed_mesh_renderer(_lib.TRIANGLE_MOLLER_TRUMBORE)
    rs = np.random.default_rng(3)
    d = rs.normal(size=(100000, 3)).astype(np.float32)
    o = (rs.uniform(-0.3, 0.3, (100000, 3))).astype(np.float32)
    rays = np.concatenate([o, d], 1)
    hw, _ = r_w.trace_rays(rays)
    hm, _ = r_m.trace_rays(rays)
    both = (hw["hit"] != 0) & (hm["hit"] != 0)
    assert both.mean() > 0.999
    same_tri = hw["tri_id"][both] == hm["tri_id"][both]
    assert same_tri.mean() > 0.999
    t_w, t_m = hw["t"][both][same_tri], hm["t"][both][same_tri]
    assert np.max(np.abs(t_w - t_m) / t_m) < 1e-5
    u_w, u_m = hw["uv"][both][same_tri], hm["uv"][both][same_tri]
    assert np.max(np.abs(u_w - u_m)) < 1e-4
    r_w.close()
    r_m.close()


def test_triangle_test_is_validated():
    r, _, _ = _closed_mesh_renderer(_lib.TRIANGLE_MOLLER_TRUMBORE)
    st = ornament.State()
    s = st.to_struct()
    s.triangle_test = 7
    with pytest.raises(_lib.OrnamentError):
        r.set_state(s)
    r.close()
