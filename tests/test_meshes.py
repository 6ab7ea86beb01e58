"""Meshes on the CPU: the OBJ loader, the mesh generators and the oracle's restatement of
MeshDistance (signed distance), RigidBody's mesh volume map and ParticleSampler.

The reference computes the point-triangle distance in FP32 from the quadratic form
Q(s, t) (MeshDistance.cpp:300-607), whose rounding error grows with the squared distance
to the triangle's first corner: near the surface of a unit-sized mesh its distances are
good to ~1e-4, so the analytic comparisons below allow that much where the true distance
is small and hold the sign exactly elsewhere.
"""
import numpy as np
import pytest

from oracle import oracle as O
from vfd_gb300 import meshes


def signed_volume(v, t):
    v = v.astype(np.float64)
    a, b, c = v[t[:, 0]], v[t[:, 1]], v[t[:, 2]]
    return float(np.einsum("ij,ij->i", a, np.cross(b, c)).sum() / 6.0)


def box_sd(p, lo, hi):
    c, h = (np.asarray(lo) + np.asarray(hi)) / 2, (np.asarray(hi) - np.asarray(lo)) / 2
    q = np.abs(np.asarray(p, np.float64) - c) - h
    return np.linalg.norm(np.maximum(q, 0), axis=1) + np.minimum(q.max(1), 0)


def test_generated_meshes_are_closed_and_outward():
    v, t = meshes.box_mesh((0, 0, 0), (1, 2, 3))
    assert signed_volume(v, t) == pytest.approx(6.0)
    v, t = meshes.icosphere((0.1, 0, 0), 1.0, 3)
    assert 0.98 * 4 / 3 * np.pi < signed_volume(v, t) < 4 / 3 * np.pi
    v, t = meshes.cone((0, 0, 0), 0.5, 1.0, 64)
    assert signed_volume(v, t) == pytest.approx(np.pi * 0.25 / 3, rel=2e-3)
    for v, t in (meshes.box_mesh((0, 0, 0), (1, 1, 1)), meshes.icosphere(subdivisions=2), meshes.cone()):
        edges = np.concatenate([t[:, [0, 1]], t[:, [1, 2]], t[:, [2, 0]]])
        fwd = {tuple(e) for e in edges}
        assert len(fwd) == len(edges) and all((b, a) in fwd for a, b in fwd)  # each edge once each way


def test_obj_loader(tmp_path):
    text = """# a unit square pyramid written by hand
o pyramid
v 0 0 0
v 1 0 0
v 1 0 1
v 0 0 1
v 0.5 1 0.5
vt 0 0
vn 0 1 0
f 1/1/1 2/1/1 3/1/1 4/1/1
f 2//1 1//1 5//1
f -4 -2 -3
f 4 3 5
f 1 5 4
o second
v 5 5 5
f 1 2 6
"""
    p = tmp_path / "pyramid.obj"
    p.write_text(text)
    v, t = meshes.load_obj(str(p))
    assert v.shape == (6, 3) and v.dtype == np.float32      # every vertex, as the reference keeps
    # the square's diagonals are equally long: split along 1-3 (tinyobjloader's quad rule)
    first = [[0, 1, 3], [1, 2, 3], [1, 0, 4], [1, 3, 2], [3, 2, 4], [0, 4, 3]]
    np.testing.assert_array_equal(t, first + [[0, 1, 5]])  # every shape (TriangleMesh)
    _, t1 = meshes.load_obj(str(p), first_shape_only=True)  # EdgeMesh(filepath)
    np.testing.assert_array_equal(t1, first)
    pq = tmp_path / "polygons.obj"
    pq.write_text("v 0 0 0\nv 2 0 0\nv 2 1 0\nv 0 1 0\nv 1 2 0\nf 1 2 3 4\nf 1 2 3 5 4\n")
    _, tq = meshes.load_obj(str(pq))
    np.testing.assert_array_equal(tq, [[0, 1, 3], [1, 2, 3], [0, 1, 2], [0, 2, 4], [0, 4, 3]])
    v2, t2 = meshes.load_obj(str(p), scale=(2, 1, 1))
    np.testing.assert_array_equal(v2[:, 0], 2 * v[:, 0])
    q = tmp_path / "box.obj"
    bv, bt = meshes.box_mesh((-1, 0, 2), (1, 0.5, 3))
    meshes.save_obj(str(q), bv, bt)
    lv, lt = meshes.load_obj(str(q))
    np.testing.assert_array_equal(lv, bv)
    np.testing.assert_array_equal(lt, bt)


def test_signed_distance_of_a_box_mesh():
    lo, hi = (-0.5, -0.25, -0.3), (0.5, 0.25, 0.3)
    v, t = meshes.box_mesh(lo, hi)
    p = np.random.default_rng(0).uniform(-1, 1, (20000, 3)).astype(np.float32)
    d = O.mesh_signed_distance(v, t, p)
    ex = box_sd(p, lo, hi)
    far = np.abs(ex) > 1e-3
    assert np.all(np.sign(d[far]) == np.sign(ex[far]))
    assert np.abs(d - ex).max() < 3e-4 and np.median(np.abs(d - ex)) < 1e-6


def test_signed_distance_of_a_sphere_mesh_and_placement():
    c, R = np.array([0.1, 0.2, 0.3]), 0.5
    v, t = meshes.icosphere(c, R, 4)
    p = np.random.default_rng(1).uniform(-1, 1, (20000, 3)).astype(np.float32)
    d = O.mesh_signed_distance(v, t, p)
    ex = np.linalg.norm(p - c, axis=1) - R
    sag = 1e-3  # the polyhedron lies within 1e-3 of the sphere at 5120 faces of radius 0.5
    assert np.abs(d - ex).max() < sag
    assert np.all(np.sign(d[np.abs(ex) > sag]) == np.sign(ex[np.abs(ex) > sag]))
    # placement: a transform applied by the oracle equals the vertices placed beforehand
    T = meshes.transform((0.25, -0.5, 1.0), (2.0, 1.0, 0.5), (10, 20, 30))
    vt = (v.astype(np.float64) @ T[:3, :3].T.astype(np.float64) + T[:3, 3]).astype(np.float32)
    np.testing.assert_allclose(O.mesh_signed_distance(v, t, p, transform=T), O.mesh_signed_distance(vt, t, p),
                               atol=2e-6)


def test_mesh_map_of_a_box_equals_the_box_map():
    r = 0.025
    v, t = meshes.box_mesh((0, 0, 0), (1.2, 0.8, 0.6))
    for inverted in (True, False):
        a = O.build_mesh_map(v, t, None, inverted, 0.0, (12, 8, 6), r)
        b = O.build_box_map((0, 0, 0), (1.2, 0.8, 0.6), inverted, 0.0, (12, 8, 6), r)
        assert a.meta() == b.meta()
        np.testing.assert_array_equal(a.cells, b.cells)
        nn = a.struct.node_count
        np.testing.assert_allclose(a.nodes[:nn], b.nodes[:nn], atol=2e-5)
        np.testing.assert_allclose(a.nodes[nn:], b.nodes[nn:], atol=1e-4 * b.nodes[nn:].max())


def _lattice(lo, hi, step):
    out, x = [], np.float32(lo)
    while x <= np.float32(hi):
        out.append(x)
        x = np.float32(x + np.float32(step))
    return np.array(out, np.float32)


def test_sampler_min_density_box_is_the_float_lattice():
    r = np.float32(0.05)
    v, t = meshes.box_mesh((0, 0, 0), (1, 0.6, 0.4))
    s = O.sample_mesh_volume(v, t, float(r), (20, 20, 20), False, 0)
    xs, ys, zs = (_lattice(0, hi, 2 * r) for hi in (1.0, 0.6, 0.4))
    Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
    lat = np.stack([X + r, Y + r, Z + r], -1).reshape(-1, 3).astype(np.float32)
    inside = box_sd(lat, (0, 0, 0), (1, 0.6, 0.4)) < -1e-4
    np.testing.assert_array_equal(s, lat[inside])
    assert len(s) == 10 * 6 * 4


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_sampler_fills_a_sphere(mode):
    r, R = 0.02, 0.3
    v, t = meshes.icosphere((0, 0, 0), R, 3)
    s = O.sample_mesh_volume(v, t, r, (20, 20, 20), False, mode)
    assert np.all(np.linalg.norm(s, axis=1) < R + 1e-3)
    assert np.all(np.diff(s[:, 2]) >= -2.0 * r)  # z is the outer loop
    # packing density of the three lattices: 1/(2r)^3, 2/(sqrt(3) 4 r^3) ... within 10 %
    vol = signed_volume(v, t)
    per = {0: 8 * r ** 3, 1: 4 * np.sqrt(3) * r ** 3, 2: 4 * np.sqrt(2) * r ** 3}[mode]
    assert len(s) == pytest.approx(vol / per, rel=0.1)
    assert len(np.unique(np.round(s / (0.01 * r)), axis=0)) == len(s)
