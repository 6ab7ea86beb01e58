"""Mesh volume maps and the mesh-volume sampler on the GPU, through the C-ABI.

* vfd_build_mesh_map of a 12-triangle box equals vfd_build_box_map of the same box:
  both distances are exact to FP32 rounding, so field 0 agrees to 2e-6 and field 1 to
  1e-5 of its maximum.
* Against the oracle's restatement of MeshDistance and RigidBody (an icosphere and a cone,
  placed by rotation, scale and translation; solid and inverted): the same grid and
  cells; field 0 with the same sign wherever |phi| > 1e-3 and equal within the FP32
  error of the reference's quadratic-form distance, which is ~4e-7 C / |d| for C the
  squared extent of the map (the GPU finds the closest point directly and is exact to
  rounding); field 1 within 2e-3 of its maximum.
* vfd_sample_mesh_volume equals the oracle's ParticleSampler bit for bit (same float
  lattice, same order) except for lattice points on the surface, where the sign of the
  interpolated distance is decided by rounding: on a box none in the min-density
  packing; in the other two packings the column at x = bounds.min.x lies on a face.
* A dam break whose container is a mesh map and whose fluid is sampled from a box mesh
  tracks the FP32 oracle given the same map, and the same scene with the box map.
"""
import numpy as np
import pytest

import vfd_gb300 as V
from oracle import oracle as O
from vfd_gb300 import meshes, scenes

pytestmark = pytest.mark.gpu


def _as_oracle(m):
    return O.VolumeMap.from_arrays(m.nodes, m.cells, m.cell_map, m.meta())


def test_mesh_map_of_a_box_equals_the_box_map():
    r = 0.025
    v, t = meshes.box_mesh((0, 0, 0), (1.2, 0.8, 0.6))
    for inverted in (True, False):
        a = V.build_mesh_map(v, t, None, inverted, 0.0, (12, 8, 6), r)
        b = V.build_box_map((0, 0, 0), (1.2, 0.8, 0.6), inverted, 0.0, (12, 8, 6), r)
        assert a.meta() == b.meta()
        np.testing.assert_array_equal(a.cells, b.cells)
        np.testing.assert_array_equal(a.cell_map, b.cell_map)
        nn = a.struct.node_count
        np.testing.assert_allclose(a.nodes[:nn], b.nodes[:nn], atol=2e-6)
        np.testing.assert_allclose(a.nodes[nn:], b.nodes[nn:], atol=1e-5 * b.nodes[nn:].max())


@pytest.mark.parametrize("shape,inverted", [("sphere", False), ("sphere", True), ("cone", False)])
def test_mesh_map_matches_oracle(shape, inverted):
    r = 0.02
    if shape == "sphere":
        v, t = meshes.icosphere((0, 0, 0), 0.3, 3)
    else:
        v, t = meshes.cone((0, 0, 0), 0.3, 0.5, 48)
    T = meshes.transform((0.4, 0.3, -0.2), (1.0, 0.8, 1.2), (15, -30, 40))
    res = (16, 14, 18)
    a = V.build_mesh_map(v, t, T, inverted, 0.01, res, r)
    b = O.build_mesh_map(v, t, T, inverted, 0.01, res, r)
    ma, mb = a.meta(), b.meta()
    for k in ("domain_min", "domain_max", "cell_size", "cell_size_inverse"):
        np.testing.assert_array_equal(ma[k], mb[k], err_msg=k)
    np.testing.assert_array_equal(a.cells, b.cells)
    nn = a.struct.node_count
    da, db = a.nodes[:nn].astype(np.float64), b.nodes[:nn].astype(np.float64)
    far = np.abs(db) > 1e-3
    assert np.all(np.sign(da[far]) == np.sign(db[far]))
    C = float(np.sum((np.asarray(ma["domain_max"]) - np.asarray(ma["domain_min"])) ** 2))
    tol = 2e-6 + 4e-7 * C / np.maximum(np.abs(db), np.sqrt(4e-7 * C))
    err = np.abs(da - db)
    print(f"{shape}: field 0 max |GPU - oracle| {err.max():.2e}, median {np.median(err):.2e}")
    assert np.all(err <= tol), (err / tol).max()
    va, vb = a.nodes[nn:], b.nodes[nn:]
    print(f"{shape}: field 1 max |GPU - oracle| {np.abs(va - vb).max():.2e} of max {vb.max():.3f}")
    assert vb.max() > 0 and np.abs(va - vb).max() < 2e-3 * vb.max()


def _compare_samples(a, b, distance, eps):
    """Equal samples in equal order, except lattice points within `eps` of the surface
    (by `distance`), where the sign of the interpolated distance is decided by rounding."""
    sa, sb = {tuple(p) for p in a.tolist()}, {tuple(p) for p in b.tolist()}
    diff = np.array(sorted(sa ^ sb), np.float32).reshape(-1, 3)
    if len(diff):
        assert np.abs(distance(diff)).max() < eps
    common = sa & sb
    keep_a = np.array([tuple(p) in common for p in a.tolist()], bool)
    keep_b = np.array([tuple(p) in common for p in b.tolist()], bool)
    np.testing.assert_array_equal(a[keep_a], b[keep_b])  # same order
    return len(diff)


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_sampler_box_matches_oracle(mode):
    # faces off the min-density lattice: no lattice point of packing 0 lies within 7e-3
    # of the surface, so that packing must agree bit for bit; packings 1 and 2 put a
    # column of points on the lower faces (x = bounds.min.x, ParticleSampler.cpp:46-60)
    v, t = meshes.box_mesh((0.1, 0.2, 0.3), (0.913, 0.717, 0.659))
    T = meshes.transform((0.5, -0.25, 0.0))
    a = V.sample_mesh_volume(v, t, 0.02, (20, 20, 20), False, mode, transform=T)
    b = O.sample_mesh_volume(v, t, 0.02, (20, 20, 20), False, mode, transform=T)
    assert len(a) > 1000
    if mode == 0:
        np.testing.assert_array_equal(a, b)
    lo, hi = np.array([0.6, -0.05, 0.3]), np.array([1.413, 0.467, 0.659])

    def box_distance(p):
        q = np.abs(p.astype(np.float64) - (lo + hi) / 2) - (hi - lo) / 2
        return np.linalg.norm(np.maximum(q, 0), axis=1) + np.minimum(q.max(1), 0)

    n = _compare_samples(a, b, box_distance, 1e-6)
    print(f"box, packing {mode}: {len(a)} GPU, {len(b)} oracle samples, {n} on the surface differ")


@pytest.mark.parametrize("mode", [0, 2])
def test_sampler_sphere_matches_oracle(mode):
    v, t = meshes.icosphere((0.05, 0.0, -0.05), 0.25, 3)
    a = V.sample_mesh_volume(v, t, 0.01, (24, 24, 24), False, mode)
    b = O.sample_mesh_volume(v, t, 0.01, (24, 24, 24), False, mode)
    n = _compare_samples(a, b, lambda p: O.mesh_signed_distance(v, t, p), 1e-3)
    print(f"sphere, packing {mode}: {len(a)} GPU, {len(b)} oracle samples, {n} differ")
    assert n < 1e-3 * len(b) + 2


def test_sampler_sizes_and_errors():
    v, t = meshes.box_mesh((0, 0, 0), (1, 1, 1))
    assert len(V.sample_mesh_volume(v, t, 0.05, (10, 10, 10), True, 0)) == 0  # inverted: nothing inside
    with pytest.raises(V.VFDError) as e:
        V.sample_mesh_volume(v, t, 0.05, (10, 10, 10), False, 3)
    assert e.value.code == V._abi.VFD_E_ARG
    with pytest.raises(V.VFDError) as e:
        V.build_mesh_map(v, np.array([[0, 1, 8]], np.uint32), None, False, 0.0, (4, 4, 4), 0.05)
    assert e.value.code == V._abi.VFD_E_ARG


def _mesh_dam_break():
    r = 0.025
    g = scenes.wall_gap(r)
    lo, hi = np.array([g, g, g]), np.array([g + 0.4, g + 0.5, g + 0.3])
    fv, ft = meshes.box_mesh(lo, hi)
    x = V.sample_mesh_volume(fv, ft, r, (20, 20, 20), False, 0)
    box = (1.2, 0.9, 0.6)
    cv, ct = meshes.box_mesh((0, 0, 0), box)
    desc = dict(ParticleRadius=r, EnableViscositySolver=0, EnableSurfaceTensionSolver=0, Viscosity=0.0,
                BoundaryViscosity=0.0, **scenes.SOLVER)
    scene = dict(x=x, v=np.zeros_like(x), desc=desc, boxes=[scenes.container((0, 0, 0), box, r, (24, 18, 12))])
    mesh_map = V.build_mesh_map(cv, ct, None, True, 0.0, (24, 18, 12), r)
    return scene, mesh_map


def test_mesh_scene_tracks_oracle_and_box_scene():
    scene, mesh_map = _mesh_dam_break()
    assert len(scene["x"]) == 8 * 10 * 6
    h = 4 * scene["desc"]["ParticleRadius"]
    g = V.scene_simulation(scene, maps=[mesh_map])
    o = O.scene_oracle(scene, 32, maps=[_as_oracle(mesh_map)])
    b = V.scene_simulation(scene)  # the analytic box map of the same container
    for k in range(5):
        sg, so = g.OnUpdate(), o.step()
        b.OnUpdate()
        assert sg["PressureSolverIterationCount"] == so["PressureSolverIterationCount"]
        xg, _, _ = g.GetState()
        xo, _, _ = o.state()
        dx = np.abs(xg - xo).max(axis=1)
        assert np.median(dx) < 1e-6 * (k + 1) ** 2 * h and dx.max() < 1e-3 * h, (np.median(dx), dx.max())
    xb, _, _ = b.GetState()
    assert np.abs(xg - xb).max() < 1e-3 * h
