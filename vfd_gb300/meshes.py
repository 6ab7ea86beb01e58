"""Triangle meshes for rigid bodies and fluid volumes.

`load_obj` reads a Wavefront OBJ as the reference's scene meshes are read
(TriangleMesh::TriangleMesh, Renderer/Mesh/TriangleMesh.cpp:40-120, through the
vendored tinyobjloader 2.0.0rc, ThirdParty/tinyobjloader): every `v` line is a vertex,
every face of every shape is kept, and a face names its corners by their position
indices (texture and normal indices are ignored; negative indices count back from the
last vertex read). `first_shape_only=True` keeps the faces of the first shape only, as
EdgeMesh::EdgeMesh(filepath) does (Renderer/Mesh/EdgeMesh.cpp:61-96); a new shape
starts at an `o` or `g` line that follows a face. Quads are split along their shorter
diagonal as tinyobjloader does (the (0,1,2),(0,2,3) pair when |v2 - v0| < |v3 - v1| in
FP32, else (0,1,3),(1,2,3)); larger polygons are split into a fan around their first
corner (tinyobjloader clips ears there; convex polygons give the same area either way).
The generators build closed meshes with outward, counter-clockwise triangles, the
orientation the signed distance expects.
"""
from __future__ import annotations

import numpy as np


def _split_polygon(idx, verts):
    if len(idx) == 3:
        return [idx]
    if len(idx) == 4:
        p = [np.asarray(verts[i], np.float32) for i in idx]
        e02, e13 = p[2] - p[0], p[3] - p[1]
        sq02 = np.float32(np.float32(e02[0] * e02[0] + e02[1] * e02[1]) + e02[2] * e02[2])
        sq13 = np.float32(np.float32(e13[0] * e13[0] + e13[1] * e13[1]) + e13[2] * e13[2])
        if sq02 < sq13:
            return [[idx[0], idx[1], idx[2]], [idx[0], idx[2], idx[3]]]
        return [[idx[0], idx[1], idx[3]], [idx[1], idx[2], idx[3]]]
    return [[idx[0], idx[k], idx[k + 1]] for k in range(1, len(idx) - 1)]


def load_obj(path: str, scale=(1.0, 1.0, 1.0), first_shape_only: bool = False):
    """(vertices float32 (n, 3), triangles uint32 (m, 3)) of an OBJ file."""
    verts, tris = [], []
    seen_face = first_done = False
    with open(path, "r", encoding="utf-8", errors="replace") as fh:
        for raw in fh:
            line = raw.split("#", 1)[0].strip()
            if not line:
                continue
            tok = line.split()
            key = tok[0]
            if key == "v":
                verts.append([np.float32(tok[1]), np.float32(tok[2]), np.float32(tok[3])])
            elif key == "f":
                if first_done:
                    continue
                if len(tok) < 4:
                    raise ValueError(f"{path}: face with fewer than three corners: {line!r}")
                idx = []
                for t in tok[1:]:
                    i = int(t.split("/", 1)[0])
                    idx.append(i - 1 if i > 0 else len(verts) + i)
                if min(idx) < 0 or max(idx) >= len(verts):
                    raise ValueError(f"{path}: face index out of range: {line!r}")
                tris += _split_polygon(idx, verts)
                seen_face = True
            elif key in ("o", "g") and seen_face and first_shape_only:
                first_done = True
    v = np.asarray(verts, np.float32).reshape(-1, 3) * np.asarray(scale, np.float32)
    t = np.asarray(tris, np.int64).reshape(-1, 3)
    return v.astype(np.float32), t.astype(np.uint32)


def save_obj(path: str, vertices, triangles) -> None:
    with open(path, "w") as fh:
        for p in np.asarray(vertices, np.float64):
            fh.write(f"v {p[0]:.9g} {p[1]:.9g} {p[2]:.9g}\n")
        for t in np.asarray(triangles, np.int64):
            fh.write(f"f {t[0] + 1} {t[1] + 1} {t[2] + 1}\n")


def box_mesh(bmin, bmax):
    """12-triangle box [bmin, bmax]."""
    lo, hi = np.asarray(bmin, np.float32), np.asarray(bmax, np.float32)
    v = np.array([[lo[0] if i & 1 == 0 else hi[0], lo[1] if i & 2 == 0 else hi[1], lo[2] if i & 4 == 0 else hi[2]]
                  for i in range(8)], np.float32)
    # per face: four corners counter-clockwise seen from outside
    quads = [(0, 4, 6, 2), (1, 3, 7, 5),  # -x, +x
             (0, 1, 5, 4), (2, 6, 7, 3),  # -y, +y
             (0, 2, 3, 1), (4, 5, 7, 6)]  # -z, +z
    t = []
    for a, b, c, d in quads:
        t += [(a, b, c), (a, c, d)]
    return v, np.asarray(t, np.uint32)


def icosphere(center=(0.0, 0.0, 0.0), radius: float = 1.0, subdivisions: int = 3):
    """Sphere of 20 * 4^subdivisions triangles, vertices on the sphere."""
    g = (1.0 + 5.0 ** 0.5) / 2.0
    v = [(-1, g, 0), (1, g, 0), (-1, -g, 0), (1, -g, 0), (0, -1, g), (0, 1, g), (0, -1, -g), (0, 1, -g),
         (g, 0, -1), (g, 0, 1), (-g, 0, -1), (-g, 0, 1)]
    v = [np.asarray(p, np.float64) / np.linalg.norm(p) for p in v]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6),
         (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10),
         (8, 6, 7), (9, 8, 1)]
    for _ in range(subdivisions):
        mid = {}

        def midpoint(a, b):
            key = (min(a, b), max(a, b))
            if key not in mid:
                m = v[a] + v[b]
                v.append(m / np.linalg.norm(m))
                mid[key] = len(v) - 1
            return mid[key]

        nf = []
        for a, b, c in f:
            ab, bc, ca = midpoint(a, b), midpoint(b, c), midpoint(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        f = nf
    verts = np.asarray(v) * radius + np.asarray(center, np.float64)
    return verts.astype(np.float32), np.asarray(f, np.uint32)


def cone(base_center=(0.0, 0.0, 0.0), radius: float = 0.5, height: float = 1.0, segments: int = 32):
    """Closed cone along +y: a disc of `segments` sides at base_center and an apex above it."""
    c = np.asarray(base_center, np.float64)
    ang = 2.0 * np.pi * np.arange(segments) / segments
    ring = np.stack([c[0] + radius * np.cos(ang), np.full(segments, c[1]), c[2] + radius * np.sin(ang)], 1)
    verts = np.vstack([ring, [c + [0.0, height, 0.0]], [c]])
    apex, bottom = segments, segments + 1
    t = []
    for i in range(segments):
        j = (i + 1) % segments
        t.append((i, apex, j))      # side, outward
        t.append((i, j, bottom))    # base, facing -y
    return verts.astype(np.float32), np.asarray(t, np.uint32)


def transform(translation=(0.0, 0.0, 0.0), scale=(1.0, 1.0, 1.0), rotation_deg=(0.0, 0.0, 0.0)):
    """4x4 placement matrix T * Rz * Ry * Rx * S (acting on column vectors)."""
    rx, ry, rz = np.radians(rotation_deg)
    cx, sx, cy, sy, cz, sz = np.cos(rx), np.sin(rx), np.cos(ry), np.sin(ry), np.cos(rz), np.sin(rz)
    Rx = np.array([[1, 0, 0], [0, cx, -sx], [0, sx, cx]])
    Ry = np.array([[cy, 0, sy], [0, 1, 0], [-sy, 0, cy]])
    Rz = np.array([[cz, -sz, 0], [sz, cz, 0], [0, 0, 1]])
    m = np.eye(4)
    m[:3, :3] = Rz @ Ry @ Rx @ np.diag(np.asarray(scale, np.float64))
    m[:3, 3] = translation
    return m.astype(np.float32)
