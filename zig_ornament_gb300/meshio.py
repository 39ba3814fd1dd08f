"""Wavefront OBJ loading for the scene API — the model path of the reference's
example app (glfw_example/examples.zig:505-577 ``loadMesh``), which imports
through assimp with Triangulate | JoinIdenticalVertices | SortByPType |
GenSmoothNormals, keeps one index stream for positions, normals and uvs,
then recentres the mesh and scales it to unit height.

``read_obj`` parses ``v`` / ``vt`` / ``vn`` / ``f`` records (polygons are fan-
triangulated, negative indices count from the end, other records are
ignored); every distinct (position, uv, normal) corner becomes one vertex, as
JoinIdenticalVertices does; meshes without normals get smooth normals (the
area-weighted face normals summed over the faces that share a position).
``load_mesh`` is ``loadMesh``: it normalises the vertices and calls
``Scene.createMesh``.
"""
from __future__ import annotations

from dataclasses import dataclass
from pathlib import Path

import numpy as np

F32 = np.float32


@dataclass
class ObjMesh:
    vertices: np.ndarray   # (n, 4) float32, w = 1
    normals: np.ndarray    # (n, 4) float32, w = 0, unit length
    uvs: np.ndarray        # (n, 2) float32, or (0, 2) without texture coordinates
    indices: np.ndarray    # (3t,) uint32, one stream for all three arrays


def _index(tok: str, count: int) -> int:
    i = int(tok)
    if i == 0:
        raise ValueError("OBJ indices start at 1")
    return i - 1 if i > 0 else count + i


def read_obj(path) -> ObjMesh:
    pos, tex, nrm = [], [], []
    corners = []   # (position, uv or -1, normal or -1) per triangle corner
    with open(path, "r", encoding="utf-8", errors="replace") as f:
        for lineno, line in enumerate(f, 1):
            parts = line.split("#", 1)[0].split()
            if not parts:
                continue
            tag = parts[0]
            try:
                if tag == "v":
                    pos.append([float(x) for x in parts[1:4]])
                elif tag == "vt":
                    tex.append([float(x) for x in (parts[1:3] + ["0"])[:2]])
                elif tag == "vn":
                    nrm.append([float(x) for x in parts[1:4]])
                elif tag == "f":
                    face = []
                    for c in parts[1:]:
                        fields = c.split("/")
                        p = _index(fields[0], len(pos))
                        t = _index(fields[1], len(tex)) if len(fields) > 1 and fields[1] else -1
                        n = _index(fields[2], len(nrm)) if len(fields) > 2 and fields[2] else -1
                        face.append((p, t, n))
                    if len(face) < 3:
                        raise ValueError("a face needs 3 corners")
                    for k in range(1, len(face) - 1):   # fan triangulation
                        corners.extend((face[0], face[k], face[k + 1]))
            except (ValueError, IndexError) as exc:
                raise ValueError(f"{path}:{lineno}: {exc}") from None
    if not corners:
        raise ValueError(f"{path}: no faces")
    c = np.array(corners, dtype=np.int64)
    P = np.array(pos, dtype=np.float64).reshape(-1, 3)
    if (c[:, 0] < 0).any() or (c[:, 0] >= len(P)).any():
        raise ValueError(f"{path}: position index out of range")
    if len(tex) and ((c[:, 1] >= len(tex)).any()):
        raise ValueError(f"{path}: uv index out of range")
    if len(nrm) and ((c[:, 2] >= len(nrm)).any()):
        raise ValueError(f"{path}: normal index out of range")
    # JoinIdenticalVertices: one vertex per distinct corner
    uniq, inverse = np.unique(c, axis=0, return_inverse=True)
    inverse = inverse.reshape(-1)
    verts = np.concatenate([P[uniq[:, 0]], np.ones((len(uniq), 1))], 1).astype(F32)
    has_uv = len(tex) > 0 and (uniq[:, 1] >= 0).all()
    uvs = np.array(tex, dtype=F32).reshape(-1, 2)[uniq[:, 1]] if has_uv else np.zeros((0, 2), F32)
    if len(nrm) > 0 and (uniq[:, 2] >= 0).all():
        N = np.array(nrm, dtype=np.float64).reshape(-1, 3)[uniq[:, 2]]
    else:
        # GenSmoothNormals: area-weighted face normals summed per position
        tri = c[:, 0].reshape(-1, 3)
        fn = np.cross(P[tri[:, 1]] - P[tri[:, 0]], P[tri[:, 2]] - P[tri[:, 0]])
        acc = np.zeros_like(P)
        for k in range(3):
            np.add.at(acc, tri[:, k], fn)
        N = acc[uniq[:, 0]]
    length = np.linalg.norm(N, axis=1, keepdims=True)
    N = np.where(length > 0, N / np.where(length > 0, length, 1.0), np.array([0.0, 1.0, 0.0]))
    normals = np.concatenate([N, np.zeros((len(N), 1))], 1).astype(F32)
    return ObjMesh(verts, normals, uvs, inverse.astype(np.uint32))


def normalize_vertices(vertices: np.ndarray) -> np.ndarray:
    """loadMesh's normalisation: centre the bounding box on the origin and
    divide by its height (max.y - min.y)."""
    v = np.asarray(vertices, dtype=F32)
    mn, mx = v[:, :3].min(axis=0), v[:, :3].max(axis=0)
    centre = mn + (mx - mn) * F32(0.5)
    height = mx[1] - mn[1]
    if not height > 0:
        raise ValueError("mesh has zero height")
    out = v.copy()
    out[:, :3] = (v[:, :3] - centre) * (F32(1.0) / height)
    return out


def load_mesh(scene, path, transform, material):
    """examples.zig loadMesh: read the OBJ, normalise, Scene.createMesh."""
    m = read_obj(Path(path))
    v = normalize_vertices(m.vertices)
    return scene.createMesh(v, m.indices, m.normals, m.indices, m.uvs, m.indices, transform, material)
