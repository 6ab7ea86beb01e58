"""The oracle's carried-state setter (test infrastructure for one-step parity along
a GPU trajectory): a run resumed from another run's carried state (positions,
velocities, viscosity warm start, temporal curvature, time step) takes the same
next step, bit for bit, in the FP32 mirror."""
import numpy as np

from oracle import oracle as O
from vfd_gb300 import _abi, scenes


def test_resumed_oracle_takes_the_same_step():
    s = scenes.small_dam_break(n_side=8, viscosity=0.02, surface_tension=0.05)
    a = O.scene_oracle(s, 32)
    for _ in range(4):
        a.step()
    x, v, _ = a.state()
    dv = a.field(_abi.FIELD_VELOCITY_DIFFERENCE)
    dk = a.field(_abi.FIELD_DELTA_FINAL_CURVATURE)
    b = O.scene_oracle(s, 32)
    b.set_carried(x, v, dv, dk, a.time_step())
    sa, sb = a.step(), b.step()
    for k in ("IterationCount", "FrameIndex"):  # counters of the run, not carried state
        sa.pop(k), sb.pop(k)
    assert sa == sb
    for u, w in zip(a.state(), b.state()):
        np.testing.assert_array_equal(u, w)
