"""Particle emission (vfd_emit, the reference has no emitter) on the GPU: appending keeps
the state of the particles already there, the appended ones take the next indices, the
run after it tracks the FP32 oracle given the same emission (in place and when the
device layout has to grow), cell-relative storage converts them, a reset goes back to
the initial particles, and the inflow emitter adds evenly spaced layers."""
import numpy as np
import pytest

import vfd_gb300 as V
from oracle import oracle as O
from vfd_gb300 import emitter, scenes

pytestmark = pytest.mark.gpu


def _maps(scene):
    r = scene["desc"]["ParticleRadius"]
    return [V.build_box_map(b["min"], b["max"], b["inverted"], b["padding"], b["resolution"], r)
            for b in scene["boxes"]]


def _pair(scene):
    maps = _maps(scene)
    g = V.scene_simulation(scene, maps=maps)
    o = O.scene_oracle(scene, 32, maps=[O.VolumeMap.from_arrays(m.nodes, m.cells, m.cell_map, m.meta())
                                        for m in maps])
    return g, o


def _drop(n_side: int, r: float, offset=(0.1, 0.5, 0.1)):
    rng = scenes.SplitMix64(11)
    x = scenes.lattice_block((n_side,) * 3, r, offset, 0.05, rng)
    v = np.tile(np.float32([0.0, -0.5, 0.0]), (len(x), 1))
    return x, v


def _compare(g, o, h, k):
    xg, vg, _ = g.GetState()
    xo, vo, _ = o.state()
    assert xg.shape == xo.shape
    dx = np.abs(xg - xo).max(axis=1)
    assert np.median(dx) < 1e-6 * (k + 1) ** 2 * h and dx.max() < 1e-3 * h, (k, np.median(dx), dx.max())


def test_emit_keeps_state_and_appends():
    s = scenes.small_dam_break(n_side=8)
    sim = V.scene_simulation(s)
    sim.Steps(3)
    x0, v0, _ = sim.GetState()
    xe, ve = _drop(3, s["desc"]["ParticleRadius"])
    sim.Emit(xe, ve)
    assert sim.GetParticleCount() == len(x0) + len(xe)
    x1, v1, _ = sim.GetState()
    np.testing.assert_array_equal(x1[:len(x0)], x0)
    np.testing.assert_array_equal(v1[:len(x0)], v0)
    np.testing.assert_array_equal(x1[len(x0):], xe)
    np.testing.assert_array_equal(v1[len(x0):], ve)
    sim.Steps(2)
    assert np.all(np.isfinite(sim.GetState()[0]))
    sim.Reset()
    assert sim.GetParticleCount() == len(x0)
    np.testing.assert_array_equal(sim.GetState()[0], s["x"])


@pytest.mark.parametrize("n_side", [2, 12])  # 343 particles in a layout of 352: 8 fit, 1728 make it grow
def test_emission_tracks_oracle(n_side):
    s = scenes.small_dam_break(n_side=7)
    g, o = _pair(s)
    h = 4 * s["desc"]["ParticleRadius"]
    for _ in range(2):
        g.OnUpdate()
        o.step()
    xe, ve = _drop(n_side, s["desc"]["ParticleRadius"], (0.25, 0.3, 0.1))
    g.Emit(xe, ve)
    o.emit(xe, ve)
    for k in range(4):
        sg, so = g.OnUpdate(), o.step()
        assert sg["PressureSolverIterationCount"] == so["PressureSolverIterationCount"]
        _compare(g, o, h, k)


def test_emit_cell_relative():
    s = scenes.small_dam_break(n_side=8)
    sim = V.scene_simulation(s)
    sim.SetPositionMode(True)
    sim.SetFluidObjects(s["x"], s["v"])
    sim.Steps(2)
    xe, ve = _drop(3, s["desc"]["ParticleRadius"])
    sim.Emit(xe, ve)
    x1, _, _ = sim.GetState()
    np.testing.assert_allclose(x1[-len(xe):], xe, atol=1e-6)
    sim.Steps(2)
    assert np.all(np.isfinite(sim.GetState()[0]))


def test_inflow_emitter_layers():
    r = 0.005
    box = (0.4, 0.6, 0.4)
    desc = dict(ParticleRadius=r, EnableViscositySolver=0, EnableSurfaceTensionSolver=0, **scenes.SOLVER)
    s = dict(x=np.zeros((0, 3), np.float32), v=np.zeros((0, 3), np.float32), desc=desc,
             boxes=[scenes.container((0, 0, 0), box, r, (16, 24, 16))])
    seed = scenes.lattice_block((4, 4, 4), r, (0.18, 0.02, 0.18), 0.0, scenes.SplitMix64(1))
    s["x"], s["v"] = seed, np.zeros_like(seed)
    sim = V.scene_simulation(s)
    em = emitter.InflowEmitter((0.2, 0.5, 0.2), (0.0, -1.0, 0.0), 0.02, 1.0, r)
    per_layer = len(em.disk)
    assert per_layer == 13  # lattice points of spacing 1 cm within 2 cm
    em.run(sim, 60)
    assert em.layers > 3 and em.emitted == em.layers * per_layer
    assert sim.GetParticleCount() == len(seed) + em.emitted
    x, v, _ = sim.GetState()
    assert np.all(np.isfinite(x)) and np.all(x > -1e-3) and np.all(x < np.array(box) + 1e-3)
    new = x[len(seed):]
    assert np.all(v[len(seed):, 1] < 0)  # the jet moves down
    first = new[:per_layer, 1].mean()
    assert first < 0.5 - 0.01  # the first layer has left the nozzle
