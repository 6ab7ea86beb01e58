"""Cell-relative positions (vfd_set_position_mode) against absolute FP32 positions and
the FP64 oracle, on a viscous dam break placed at the origin and translated by about a
kilometre: absolute FP32 coordinates lose their low bits far from the origin, the
cell-relative form does not. GPU and oracle start from the same FP32 inputs and use the
same volume map, so the difference after 20 steps is the FP32 arithmetic's."""
import numpy as np
import pytest

import vfd_gb300 as V
from oracle import oracle as O
from vfd_gb300 import scenes

pytestmark = pytest.mark.gpu

STEPS = 20
SHIFT = np.array([1000.0, 200.0, -300.0])


def _scene(shift):
    s = scenes.small_dam_break(n_side=10, viscosity=0.02, seed=5)
    x = (s["x"].astype(np.float64) + shift)
    b = s["boxes"][0]
    box = (tuple(np.array(b["min"]) + shift), tuple(np.array(b["max"]) + shift))
    return x, s["desc"], box, b


def _run(shift, cell_rel):
    x, desc, box, b = _scene(shift)
    r = desc["ParticleRadius"]
    m = O.build_box_map(box[0], box[1], b["inverted"], b["padding"], b["resolution"], r)
    sim = V.DFSPHSimulation(V.make_desc(**desc))
    sim.SetPositionMode(cell_rel)
    sim.SetFluidObjects(x.astype(np.float32), np.zeros_like(x, dtype=np.float32))
    sim.AddRigidBody(m)
    sim.Steps(STEPS)
    xg, _, _ = sim.GetState()
    orc = O.OracleSim(V.make_desc(**desc), 64)
    orc.set_fluid(x.astype(np.float32), np.zeros_like(x, dtype=np.float32))
    orc.add_rigid_body(m)
    for _ in range(STEPS):
        orc.step()
    xo, _, _ = orc.state()
    return xg.astype(np.float64), xo, np.abs(xg.astype(np.float64) - xo).max()


@pytest.fixture(scope="module")
def runs():
    out = {}
    for name, shift in (("origin", np.zeros(3)), ("far", SHIFT)):
        for mode in (False, True):
            out[(name, mode)] = _run(shift, mode)
            print(f"{name:6s} {'cell-relative' if mode else 'absolute':13s}: max |x - x_FP64| after {STEPS} steps "
                  f"= {out[(name, mode)][2]:.3e} m")
    return out


def test_cell_relative_matches_absolute_near_the_origin(runs):
    e_abs, e_rel = runs[("origin", False)][2], runs[("origin", True)][2]
    assert e_rel < 2.0 * e_abs + 1e-6


def test_cell_relative_keeps_its_accuracy_far_from_the_origin(runs):
    e_abs0 = runs[("origin", False)][2]
    e_abs_far, e_rel_far = runs[("far", False)][2], runs[("far", True)][2]
    assert e_rel_far < 3.0 * e_abs0 + 1e-6
    assert e_abs_far > 3.0 * e_rel_far
