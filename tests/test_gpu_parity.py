"""Parity of the CUDA DFSPH step with the CPU oracle, through the C-ABI.

Bit-exact: cell keys, sort permutation, neighbour counts, offsets and lists
(against the FP32 oracle, whose distance test rounds like the kernel's).
Tolerances (FP32 kernel vs oracle, same inputs):
  * one step from the same state, against the FP32 oracle: density rel 1e-6
    (median; 99th percentile 1e-5, max 1e-3 where a boundary sample's kernel-table
    index flips), factor rel 1e-5 (median), positions 1e-6 h, velocities 1e-4 m/s
    (median; the tail is bounded by 1e-3 h for discrete branches such as a
    neighbour at exactly h);
  * against the FP64 oracle after 20 steps: median position error 1e-3 h,
    kinetic energy and mean density within 1 %.
"""
import numpy as np
import pytest

import vfd_gb300 as V
from oracle import oracle as O
from vfd_gb300 import _abi, scenes

pytestmark = pytest.mark.gpu


def gpu_maps(scene):
    r = scene["desc"]["ParticleRadius"]
    return [V.build_box_map(b["min"], b["max"], b["inverted"], b["padding"], b["resolution"], r)
            for b in scene["boxes"]]


def as_oracle_maps(maps):
    return [O.VolumeMap.from_arrays(m.nodes, m.cells, m.cell_map, m.meta()) for m in maps]


def pair(scene, precision=32, overrides=None):
    maps = gpu_maps(scene)
    g = V.scene_simulation(scene, overrides, maps=maps)
    o = O.scene_oracle(scene, precision, overrides, maps=as_oracle_maps(maps))
    return g, o


def assert_neighbors_equal(g, o):
    a = g.GetNeighbors()
    b = o.neighbors()
    for k in ("counts", "offsets", "sort_indices", "cell_keys"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    np.testing.assert_array_equal(a["list"], b["list"])


@pytest.mark.parametrize("factory", [
    lambda: scenes.small_dam_break(n_side=12),
    lambda: scenes.dam_break_8k(),
    lambda: scenes.viscous_dam_break(n_side=40),
])
def test_search_bit_exact(factory):
    s = factory()
    g = V.scene_simulation(s)
    o = O.scene_oracle(s, 32, maps=[])
    g.FindNeighbors()
    o.find_neighbors()
    assert_neighbors_equal(g, o)


@pytest.mark.parametrize("n,side", [(3000, 2.5), (600, 1.2)])
def test_search_bit_exact_dense_cells(n, side):
    # cells of 100+ particles (the warp-per-cell search then takes a cell's particles
    # 32 at a time) and particles past the 70-neighbour cap, beside a normal block
    s = scenes.small_dam_break(n_side=8)
    h = 4 * s["desc"]["ParticleRadius"]
    rng = np.random.default_rng(n)
    blob = (np.float32([0.6, 0.3, 0.3]) + side * h * rng.random((n, 3))).astype(np.float32)
    x = np.concatenate([s["x"], blob]).astype(np.float32)
    s = dict(s, x=x, v=np.zeros_like(x))
    g = V.scene_simulation(s)
    o = O.scene_oracle(s, 32, maps=[])
    g.FindNeighbors()
    o.find_neighbors()
    a = g.GetNeighbors()
    assert a["counts"].max() == 70 and a["counts"].min() < 70
    assert_neighbors_equal(g, o)


def test_search_bit_exact_after_steps():
    s = scenes.small_dam_break(n_side=14)
    g = V.scene_simulation(s)
    for _ in range(15):
        g.OnUpdate()
    x, v, _ = g.GetState()
    o = O.OracleSim(_abi.make_desc(**s["desc"]), 32)
    o.set_fluid(x, v)
    o.find_neighbors()
    g.FindNeighbors()
    assert_neighbors_equal(g, o)


def test_box_map_matches_oracle():
    r = 0.025
    a = V.build_box_map((0, 0, 0), (1.2, 0.8, 0.6), True, 0.0, (12, 8, 6), r)
    b = O.build_box_map((0, 0, 0), (1.2, 0.8, 0.6), True, 0.0, (12, 8, 6), r)
    nn = a.struct.node_count
    np.testing.assert_array_equal(a.cells, b.cells)
    np.testing.assert_array_equal(a.cell_map, b.cell_map)
    np.testing.assert_allclose(a.nodes[:nn], b.nodes[:nn], rtol=0, atol=1e-6)
    vol = b.nodes[nn:]
    np.testing.assert_allclose(a.nodes[nn:], vol, rtol=0, atol=1e-5 * vol.max())


def _compare_step(g, o, h, median_tol=1e-6):
    sg, so = g.OnUpdate(), o.step()
    for k in ("PressureSolverIterationCount", "DivergenceSolverIterationCount", "ViscositySolverIterationCount"):
        assert sg[k] == so[k], (k, sg[k], so[k])
    assert sg["TimeStepSize"] == pytest.approx(so["TimeStepSize"], rel=1e-6)
    xg, vg, ag = g.GetState()
    xo, vo, ao = o.state()
    dx = np.abs(xg - xo).max(axis=1)
    dv = np.abs(vg - vo).max(axis=1)
    assert np.median(dx) < median_tol * h and dx.max() < 1e-3 * h, (np.median(dx), dx.max())
    assert np.median(dv) < 1e-4, np.median(dv)
    return sg, so


def test_one_step_fields_match_fp32_oracle():
    s = scenes.small_dam_break(n_side=12)
    g, o = pair(s, 32)
    h = 4 * s["desc"]["ParticleRadius"]
    _compare_step(g, o, h)
    rho_g, rho_o = g.GetField(_abi.FIELD_DENSITY), o.field(_abi.FIELD_DENSITY)
    rel = np.abs(rho_g / rho_o - 1)
    # a boundary sample's table index can flip with rounding (its volume is ~30 particle
    # volumes, so one table step moves the density by ~1e-4)
    assert np.median(rel) < 1e-6 and np.quantile(rel, 0.99) < 1e-5 and rel.max() < 1e-3
    fg, fo = g.GetField(_abi.FIELD_FACTOR), o.field(_abi.FIELD_FACTOR)
    relf = np.abs(fg - fo) / np.maximum(np.abs(fo), 1e-30)
    assert np.median(relf) < 1e-5 and np.quantile(relf, 0.99) < 1e-3
    vb_g, vb_o = g.GetField(_abi.FIELD_BOUNDARY_VOLUME), o.field(_abi.FIELD_BOUNDARY_VOLUME)
    np.testing.assert_allclose(vb_g, vb_o, rtol=1e-4, atol=1e-7 * max(1e-12, vb_o.max()))


def test_steps_track_fp32_oracle():
    s = scenes.small_dam_break(n_side=12)
    g, o = pair(s, 32)
    h = 4 * s["desc"]["ParticleRadius"]
    for k in range(5):
        # rounding differences grow by a few ulp of the position per step
        _compare_step(g, o, h, median_tol=1e-6 * (k + 1) ** 2)


@pytest.mark.parametrize("name", ["plain", "viscous", "surface_tension", "dam_break_8k", "viscous_dam_break_64k",
                                  "viscous_drop_33k"])
def test_cuda_step_equals_reference_kernels(name):
    """The CUDA step against the reference's own step kernels (DFSPHKernels.cu compiled for
    the CPU, tests/golden/ref_step.npz; see tests/test_ref_step_golden.py): five steps of
    three 1,000-particle dam breaks and three benchmark workloads from the same inputs and
    volume maps. Iteration counts and time steps as for the oracle; positions within 2.5e-5 h
    at the median and 1e-3 h at the maximum, the bounds of the CUDA step against the FP32
    oracle over five steps (0.05 h at the maximum with surface tension at 64k particles,
    where a surface particle's Monte-Carlo coverage test can flip, as against the oracle)."""
    import test_ref_step_golden as T

    scene = T.M.cases()[name]
    g = V.scene_simulation(scene, maps=T.M.box_maps(scene))

    def state():
        x, v, _ = g.GetState()
        return x, v

    pos_max = 0.05 if name == "viscous_dam_break_64k" else 1e-3
    T.check_against_fixture(name, scene, g.OnUpdate, state, g.GetField, pos_median=2.5e-5, pos_max=pos_max)


def test_empty_fluid_steps_and_returns_an_empty_state():
    s = scenes.small_dam_break(n_side=4)
    s["x"] = np.zeros((0, 3), np.float32)
    s["v"] = np.zeros((0, 3), np.float32)
    g = V.scene_simulation(s)
    g.Steps(3)
    g.OnUpdate()
    x, v, a = g.GetState()
    assert x.shape == v.shape == a.shape == (0, 3)
    assert g.GetParticleCount() == 0


@pytest.mark.parametrize("where", ["free", "wall"])
def test_single_particle_matches_fp32_oracle(where):
    """One particle: no fluid neighbours, density below rest, so both solves stop at
    their minimum iteration count; near the floor and the back wall the volume map
    pushes it away (the boundary density and gradient paths with nothing else)."""
    s = scenes.small_dam_break(n_side=4)
    r = s["desc"]["ParticleRadius"]
    y = 0.15 if where == "free" else scenes.wall_gap(r) + 1.2 * r
    s["x"] = np.array([[0.2, y, 0.1]], np.float32)
    s["v"] = np.zeros_like(s["x"])
    g, o = pair(s, 32)
    h = 4 * r
    for _ in range(8):
        sg, so = g.OnUpdate(), o.step()
        for k in ("PressureSolverIterationCount", "DivergenceSolverIterationCount"):
            assert sg[k] == so[k], (k, sg[k], so[k])
        assert sg["TimeStepSize"] == pytest.approx(so["TimeStepSize"], rel=1e-6)
        xg, vg, _ = g.GetState()
        xo, vo, _ = o.state()
        assert xg.shape == (1, 3)
        assert np.abs(xg - xo).max() < 1e-5 * h, (xg, xo)
        assert np.abs(vg - vo).max() < 1e-4, (vg, vo)


def test_twenty_steps_track_fp64_oracle():
    s = scenes.dam_break_8k(n_side=12, box_scale=(2, 1, 1))
    g, o = pair(s, 64)
    h = 4 * s["desc"]["ParticleRadius"]
    for _ in range(20):
        sg, so = g.OnUpdate(), o.step()
        assert sg["PressureSolverError"] <= 1.0 + 1e-6
    xg, vg, _ = g.GetState()
    xo, vo, _ = o.state()
    dx = np.linalg.norm(xg - xo, axis=1)
    assert np.median(dx) < 1e-3 * h, np.median(dx)
    ke_g, ke_o = (vg.astype(np.float64) ** 2).sum(), (vo ** 2).sum()
    assert ke_g == pytest.approx(ke_o, rel=1e-2)
    assert g.GetField(_abi.FIELD_DENSITY).mean() == pytest.approx(o.field(_abi.FIELD_DENSITY).mean(), rel=1e-2)


def test_viscosity_cg_matches_oracle():
    s = scenes.small_dam_break(n_side=12, viscosity=0.05)
    g, o = pair(s, 32)
    h = 4 * s["desc"]["ParticleRadius"]
    iters = []
    for k in range(3):
        sg, so = _compare_step(g, o, h, median_tol=1e-6 * (k + 1) ** 2)
        iters.append(sg["ViscositySolverIterationCount"])
        assert sg["ViscositySolverError"] == pytest.approx(so["ViscositySolverError"], rel=1e-2, abs=1e-6)
    # the first step starts at rest: b = v = 0 takes the reference's |b|^2 == 0 exit
    assert iters[0] == 0 and min(iters[1:]) > 0
    ddv = np.abs(g.GetField(_abi.FIELD_VELOCITY_DIFFERENCE) - o.field(_abi.FIELD_VELOCITY_DIFFERENCE)).max(axis=1)
    # particles next to the wall see the boundary term in matrix form (other rounding)
    assert np.quantile(ddv, 0.995) < 1e-4 and ddv.max() < 1e-3


def test_surface_tension_matches_oracle():
    s = scenes.small_dam_break(n_side=12, surface_tension=0.05)
    g, o = pair(s, 32, dict(CSD=10000, CSDFix=-1))
    h = 4 * s["desc"]["ParticleRadius"]
    for k in range(2):
        sg, so = _compare_step(g, o, h, median_tol=1e-6 * (k + 1) ** 2)
        assert sg["SurfaceTensionSampleCount"] == so["SurfaceTensionSampleCount"]
    ng, no = g.GetField(_abi.FIELD_SURFACE_NORMAL), o.field(_abi.FIELD_SURFACE_NORMAL)
    surf_g = np.any(ng != 0, axis=1)
    surf_o = np.any(no != 0, axis=1)
    assert surf_o.sum() > 0
    assert np.mean(surf_g == surf_o) > 0.995
    both = surf_g & surf_o
    assert np.median(np.abs(ng[both] - no[both]).max(axis=1)) < 1e-4


def test_graph_mode_equals_eager_mode():
    s = scenes.small_dam_break(n_side=10, viscosity=0.01, surface_tension=0.05)
    maps = gpu_maps(s)
    a = V.scene_simulation(s, maps=maps)
    b = V.scene_simulation(s, maps=maps)
    b.SetGraphMode(False)
    for _ in range(6):
        sa, sb = a.OnUpdate(), b.OnUpdate()
        assert sa == sb
    for u, w in zip(a.GetState(), b.GetState()):
        np.testing.assert_array_equal(u, w)


def test_grid_growth_keeps_parity():
    """Particles flying apart outgrow the initial cell table; the step is redone."""
    rng = scenes.SplitMix64(5)
    r = 0.025
    x = scenes.lattice_block((8, 8, 8), r, (0, 0, 0), 0.05, rng)
    c = x.mean(axis=0)
    v = (x - c) * 40.0
    desc = dict(ParticleRadius=r, EnableViscositySolver=0, EnableSurfaceTensionSolver=0, Gravity=(0, 0, 0),
                **scenes.SOLVER)
    s = dict(x=x, v=v.astype(np.float32), desc=desc, boxes=[])
    g, o = pair(s, 32)
    for _ in range(12):
        g.OnUpdate()
        o.step()
    xg, _, _ = g.GetState()
    xo, _, _ = o.state()
    assert np.median(np.abs(xg - xo)) < 1e-5
    g.FindNeighbors()
    o2 = O.OracleSim(_abi.make_desc(**desc), 32)
    o2.set_fluid(xg, None)
    o2.find_neighbors()
    assert_neighbors_equal(g, o2)


def test_batch_matches_single_scenes():
    sc = [scenes.small_dam_break(n_side=n, viscosity=vv, seed=sd) for n, vv, sd in
          [(8, 0.0, 1), (11, 0.02, 2), (9, 0.2, 3)]]
    maps = [gpu_maps(s) for s in sc]
    batch = V.DFSPHSimulation(scenes=[_abi.make_desc(**s["desc"]) for s in sc])
    for k, s in enumerate(sc):
        batch.SetFluidObjects(s["x"], s["v"], scene=k)
        for m in maps[k]:
            batch.AddRigidBody(m, scene=k)
    singles = [V.scene_simulation(s, maps=maps[k]) for k, s in enumerate(sc)]
    for _ in range(4):
        batch.Steps(1)
        for one in singles:
            one.OnUpdate()
    for k, one in enumerate(singles):
        xb, vb, _ = batch.GetState(scene=k)
        xs, vs, _ = one.GetState()
        np.testing.assert_allclose(xb, xs, atol=1e-6)
        np.testing.assert_allclose(vb, vs, atol=1e-5)
        assert batch.GetDebugInfo(scene=k)["PressureSolverIterationCount"] == \
            one.GetDebugInfo()["PressureSolverIterationCount"]


def test_non_finite_input_is_rejected():
    s = scenes.small_dam_break(n_side=4)
    x = s["x"].copy()
    x[3, 1] = np.nan
    sim = V.DFSPHSimulation(_abi.make_desc(**s["desc"]))
    with pytest.raises(V.VFDError) as e:
        sim.SetFluidObjects(x)
    assert e.value.code == _abi.VFD_E_NAN


def test_simulate_emits_frames():
    s = scenes.small_dam_break(n_side=6)
    sim = V.scene_simulation(s, dict(FrameCount=3, FrameLength=0.004))
    seen = []
    n = sim.Simulate(lambda i, x, v, a, mv, dt: seen.append((i, x.shape)))
    assert n == 3 and [f[0] for f in seen] == [0, 1, 2]
    assert all(f[1] == (len(s["x"]), 3) for f in seen)


def test_autotune_restores_state_and_keeps_parity():
    s = scenes.small_dam_break(n_side=10, viscosity=0.02)
    maps = gpu_maps(s)
    a = V.scene_simulation(s, maps=maps)
    b = V.scene_simulation(s, maps=maps)
    a.OnUpdate()
    b.OnUpdate()
    before = a.GetState()
    lanes = a.Autotune(2)
    assert set(lanes.values()) <= {4, 8, 16}
    for u, w in zip(before, a.GetState()):
        np.testing.assert_array_equal(u, w)
    b.SetLanes(a.GetLanes())
    for _ in range(3):
        assert a.OnUpdate() == b.OnUpdate()
    for u, w in zip(a.GetState(), b.GetState()):
        np.testing.assert_array_equal(u, w)


@pytest.mark.parametrize("lanes", [4, 8, 16])
def test_lane_counts_agree(lanes):
    s = scenes.small_dam_break(n_side=10, viscosity=0.02, surface_tension=0.05)
    g, o = pair(s, 32)
    g.SetLanes([lanes] * len(V.TUNED_KERNELS))
    h = 4 * s["desc"]["ParticleRadius"]
    for k in range(2):
        _compare_step(g, o, h, median_tol=1e-6 * (k + 1) ** 2)
    g.FindNeighbors()
    o2 = O.OracleSim(_abi.make_desc(**s["desc"]), 32)
    o2.set_fluid(g.GetState()[0], None)
    o2.find_neighbors()
    assert_neighbors_equal(g, o2)


def test_search_equals_reference_kernels():
    """The GPU search against the reference's own ParticleSearchKernels.cu (run on the CPU
    by tests/golden/make_ref_search.py; digests in tests/golden/ref_search.json): counts,
    offsets, the CSR list, the sort permutation and the cell keys, bit for bit, on the
    8k and 64k dam breaks, dense cells past the 70-neighbour cap and a uniform cloud."""
    import hashlib
    import json
    import os
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.join(here, "golden"))
    import make_ref_search as M
    golden = json.load(open(os.path.join(here, "golden", "ref_search.json")))["cases"]
    for name, (x, h) in M.cases().items():
        g = V.DFSPHSimulation(_abi.make_desc(ParticleRadius=h / 4))
        g.SetFluidObjects(x)
        g.FindNeighbors()
        a = g.GetNeighbors()
        got = {k: hashlib.sha256(np.ascontiguousarray(a[k], np.uint32).tobytes()).hexdigest()
               for k in golden[name]["sha256"]}
        assert got == golden[name]["sha256"], name
        g.close()


@pytest.mark.parametrize("tiles", [1, 3, 4])
def test_tile_passes_match_oracle(tiles):
    """The other forms of the solver-loop passes -- neighbour rows with gradW / r formed from
    the table per pair (1), cell tiles of 2x2x2 or 4x2x2 cells staged in shared memory,
    neighbours walked by stencil position (3, 4) -- hold the same one-step tolerances
    against the FP32 oracle as the neighbour-row passes, with viscosity and surface
    tension on."""
    s = scenes.small_dam_break(n_side=12, viscosity=0.02, surface_tension=0.05)
    g, o = pair(s, 32)
    g.SetTiles([tiles] * len(V.TUNED_KERNELS))
    assert set(g.GetTiles().values()) == {tiles}
    h = 4 * s["desc"]["ParticleRadius"]
    for k in range(3):
        _compare_step(g, o, h, median_tol=1e-6 * (k + 1) ** 2)


def test_tile_passes_in_a_batch_match_single_scenes():
    sc = [scenes.small_dam_break(n_side=n, viscosity=vv, seed=sd) for n, vv, sd in
          [(8, 0.0, 1), (11, 0.02, 2), (9, 0.2, 3)]]
    maps = [gpu_maps(s) for s in sc]
    batch = V.batch_simulation(sc, maps)
    batch.SetTiles([3] * len(V.TUNED_KERNELS))
    singles = [V.scene_simulation(s, maps=maps[k]) for k, s in enumerate(sc)]
    for one in singles:
        one.SetTiles([3] * len(V.TUNED_KERNELS))
    for _ in range(4):
        batch.Steps(1)
        for one in singles:
            one.OnUpdate()
    for k, one in enumerate(singles):
        xb, vb, _ = batch.GetState(scene=k)
        xs, vs, _ = one.GetState()
        np.testing.assert_allclose(xb, xs, atol=1e-6)
        np.testing.assert_allclose(vb, vs, atol=1e-5)


@pytest.mark.parametrize("block", [64, 256])
def test_block_sizes_agree(block):
    """Other block sizes of the neighbour-row kernels (the autotuner's choices) keep the
    one-step tolerances against the FP32 oracle."""
    s = scenes.small_dam_break(n_side=10, viscosity=0.02, surface_tension=0.05)
    g, o = pair(s, 32)
    g.SetBlocks([block] * len(V.TUNED_KERNELS))
    assert set(g.GetBlocks().values()) == {block}
    h = 4 * s["desc"]["ParticleRadius"]
    for k in range(2):
        _compare_step(g, o, h, median_tol=1e-6 * (k + 1) ** 2)
