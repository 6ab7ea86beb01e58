"""vfd_simulate's asynchronous frame pipeline (steps queued ahead of the host, frames
copied to pinned memory on a second stream) against the synchronous frame loop of the
reference (DFSPHImplementation.cu:52-55, one step at a time, the state read when the
frame index advances): the same frames bit for bit, the run ending on the step that
completed the last frame, also when the search grid outgrows its cell table mid-run
and in eager (graph-less) mode."""
import numpy as np
import pytest

import vfd_gb300 as V
from vfd_gb300 import scenes

pytestmark = pytest.mark.gpu


def _synchronous(scene, overrides, graph=True):
    sim = V.scene_simulation(scene, overrides)
    sim.SetGraphMode(graph)
    frames, last, steps = [], 0, 0
    while last < overrides["FrameCount"]:
        st = sim.OnUpdate()
        steps += 1
        if st["FrameIndex"] != last:
            last = st["FrameIndex"]
            frames.append(sim.GetState())
    return frames, steps


def _asynchronous(scene, overrides, graph=True):
    sim = V.scene_simulation(scene, overrides)
    sim.SetGraphMode(graph)
    got = []
    n = sim.Simulate(lambda i, x, v, a, mv, dt: got.append((i, x, v, a)))
    assert n == overrides["FrameCount"] == len(got)
    assert [g[0] for g in got] == list(range(n))
    return sim, got


def _assert_same(ref, got, sim):
    for (xr, vr, ar), (_, x, v, a) in zip(ref, got):
        np.testing.assert_array_equal(x, xr)
        np.testing.assert_array_equal(v, vr)
        np.testing.assert_array_equal(a, ar)
    x, v, a = sim.GetState()  # the run ends on the last frame's step
    np.testing.assert_array_equal(x, ref[-1][0])
    np.testing.assert_array_equal(v, ref[-1][1])


@pytest.mark.parametrize("graph", [True, False])
def test_frames_equal_synchronous_loop(graph):
    s = scenes.small_dam_break(n_side=8, viscosity=0.01)
    ov = dict(FrameCount=6, FrameLength=0.006, MaxTimeStepSize=0.002)
    ref, steps = _synchronous(s, ov, graph)
    assert steps > ov["FrameCount"]  # several steps per frame
    sim, got = _asynchronous(s, ov, graph)
    _assert_same(ref, got, sim)
    # a second run starts again from the initial particles
    sim2_frames = []
    sim.Simulate(lambda i, x, v, a, mv, dt: sim2_frames.append(x))
    np.testing.assert_array_equal(sim2_frames[0], ref[0][0])


def test_frames_through_grid_growth():
    rng = scenes.SplitMix64(5)
    r = 0.025
    x = scenes.lattice_block((8, 8, 8), r, (0, 0, 0), 0.05, rng)
    v = (x - x.mean(axis=0)) * 40.0
    desc = dict(ParticleRadius=r, EnableViscositySolver=0, EnableSurfaceTensionSolver=0, Gravity=(0, 0, 0),
                **scenes.SOLVER)
    s = dict(x=x, v=v.astype(np.float32), desc=desc, boxes=[])
    ov = dict(FrameCount=8, FrameLength=0.0005)
    ref, _ = _synchronous(s, ov)
    sim, got = _asynchronous(s, ov)
    _assert_same(ref, got, sim)


def test_zero_frames_and_continuation():
    s = scenes.small_dam_break(n_side=6)
    sim = V.scene_simulation(s, dict(FrameCount=0))
    assert sim.Simulate(lambda *a: None) == 0
    sim = V.scene_simulation(s, dict(FrameCount=2, FrameLength=0.002))
    sim.Simulate()
    st = sim.OnUpdate()  # stepping goes on after the run (no stop word left behind)
    assert st["PressureSolverIterationCount"] > 0
