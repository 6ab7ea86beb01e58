"""Failure handling of the step on the GPU, made on the host side only (no kernel
is driven into a fault or an endless loop):

* solvers forced not to converge (an iteration cap of 1-2 with an unreachable
  tolerance) stop at their caps inside the CUDA graph and in eager mode, report
  VFD_FLAG_*_CAP, and the step returns VFD_OK with the state finite;
* non-finite input is rejected with VFD_E_NAN before it reaches the device;
* checkpoints: a run restored from a checkpoint repeats the original run bit for
  bit, and a mismatched image is refused with a status code.
"""
import numpy as np
import pytest

import vfd_gb300 as V
from vfd_gb300 import _abi, scenes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("graph", [True, False])
def test_pressure_cap_is_flagged_and_the_step_returns(graph):
    s = scenes.small_dam_break(n_side=10)
    sim = V.scene_simulation(s, dict(MinPressureSolverIterations=1, MaxPressureSolverIterations=1,
                                     MaxPressureSolverError=1e-6))
    sim.SetGraphMode(graph)
    sim.Steps(2)
    st = sim.OnUpdate()
    assert st["PressureSolverIterationCount"] == 1
    assert st["Flags"] & _abi.VFD_FLAG_PRESSURE_CAP
    assert np.isfinite(sim.GetState()[0]).all()


@pytest.mark.parametrize("graph", [True, False])
def test_divergence_cap_is_flagged(graph):
    s = scenes.small_dam_break(n_side=10)
    sim = V.scene_simulation(s, dict(MinDivergenceSolverIterations=1, MaxDivergenceSolverIterations=1,
                                     MaxDivergenceSolverError=1e-9))
    sim.SetGraphMode(graph)
    sim.Steps(3)
    st = sim.OnUpdate()
    assert st["DivergenceSolverIterationCount"] == 1
    assert st["Flags"] & _abi.VFD_FLAG_DIVERGENCE_CAP


@pytest.mark.parametrize("graph", [True, False])
def test_viscosity_cap_is_flagged(graph):
    s = scenes.small_dam_break(n_side=10, viscosity=0.05)
    sim = V.scene_simulation(s, dict(MaxViscositySolverIterations=2, MaxViscositySolverError=1e-12))
    sim.SetGraphMode(graph)
    sim.Steps(3)
    st = sim.OnUpdate()
    assert st["ViscositySolverIterationCount"] == 2
    assert st["Flags"] & _abi.VFD_FLAG_VISCOSITY_CAP
    assert np.isfinite(sim.GetState()[1]).all()


def test_non_finite_state_is_rejected():
    s = scenes.small_dam_break(n_side=6)
    sim = V.scene_simulation(s)
    sim.Steps(1)
    x, v, _ = sim.GetState()
    v[5, 0] = np.inf
    with pytest.raises(V.VFDError) as e:
        sim.SetState(x, v)
    assert e.value.code == _abi.VFD_E_NAN


@pytest.mark.parametrize("graph", [True, False])
def test_restore_repeats_the_run(graph):
    """Carried state x, v, viscosity warm start, temporal curvature, dt and the frame
    clock; a fresh simulation of the same scene restored from the image continues
    exactly as the original."""
    s = scenes.small_dam_break(n_side=10, viscosity=0.02, surface_tension=0.05)
    a = V.scene_simulation(s)
    a.SetGraphMode(graph)
    a.Steps(4)
    image = a.Checkpoint()
    a.Steps(3)
    xa, va, aa = a.GetState()
    sa = a.GetDebugInfo()
    b = V.scene_simulation(s)
    b.SetGraphMode(graph)
    b.Steps(1)  # a different state and clock, overwritten by the image
    b.Restore(image)
    b.Steps(3)
    for u, w in zip((xa, va, aa), b.GetState()):
        np.testing.assert_array_equal(u, w)
    sb = b.GetDebugInfo()
    for k in ("TimeStepSize", "PressureSolverIterationCount", "ViscositySolverIterationCount", "FrameTime"):
        assert sa[k] == sb[k], k
    # the same simulation, rewound
    a.Restore(image)
    a.Steps(3)
    np.testing.assert_array_equal(a.GetState()[0], xa)


def test_restore_refuses_a_mismatched_image():
    a = V.scene_simulation(scenes.small_dam_break(n_side=6))
    a.Steps(1)
    image = a.Checkpoint()
    b = V.scene_simulation(scenes.small_dam_break(n_side=7))
    with pytest.raises(V.VFDError) as e:
        b.Restore(image)
    assert e.value.code == _abi.VFD_E_STATE
    with pytest.raises(V.VFDError) as e:
        a.Restore(image[:40])
    assert e.value.code == _abi.VFD_E_ARG
