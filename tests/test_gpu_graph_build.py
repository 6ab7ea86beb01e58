"""The step graph has one conditional while node per solver loop it runs (divergence,
viscosity CG, pressure). It must build, and the steps must run from it rather than from
host launches, whichever loops the scene leaves out: a conditional handle that no node
uses makes the graph's instantiation fail, and the library would then quietly launch
the same kernels from the host."""
import numpy as np
import pytest

import vfd_gb300 as V
from vfd_gb300 import scenes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("div,visc", [(1, 1), (0, 1), (1, 0), (0, 0)])
def test_step_graph_builds_for_every_solver_set(div, visc):
    s = scenes.viscous_drop_33k(r=0.006)
    over = dict(EnableDivergenceSolverError=div, EnableViscositySolver=visc)
    g = V.scene_simulation(s, desc_overrides=over)
    g.Steps(3)
    assert g.GetGraphMode() == (True, True)
    e = V.scene_simulation(s, desc_overrides=over)
    e.SetGraphMode(False)
    e.Steps(3)
    assert e.GetGraphMode() == (False, False)
    np.testing.assert_array_equal(g.GetState()[0], e.GetState()[0])


def test_recording_and_adjoint_graphs_build():
    # the adjoint's recording steps and its CG solve are graphs too (divergence solve off,
    # as in the smooth variant that the gradient checks use)
    s = scenes.viscous_drop_33k(r=0.006)
    sim = V.scene_simulation(s, desc_overrides=dict(EnableDivergenceSolverError=0))
    sim.AdjointForward(6, 3)
    x, v, _ = sim.GetState()
    sim.AdjointBackward(np.ones_like(x) * 1e-3, np.zeros_like(v))
    assert sim.GetGraphMode() == (True, True)


def test_kernel_profile_covers_the_step():
    # vfd_profile_kernels times every kernel of the step with CUDA events: the once-per-step
    # kernels appear once per step, the solver loops once per iteration
    s = scenes.small_dam_break(n_side=12)
    sim = V.scene_simulation(s)
    sim.Steps(2)
    prof = sim.ProfileKernels(3)
    for k in ("k_neighbors", "k_boundary", "k_density_factor", "k_pres_init", "k_ctrl_end"):
        assert k in prof and prof[k][0] == 3 and prof[k][1] > 0.0, (k, prof.get(k))
    assert prof["k_jacobi_iter"][0] == prof["k_pressure_accel"][0] >= 3
    assert sim.GetGraphMode() == (True, True)  # profiling runs eagerly but leaves graphs on
