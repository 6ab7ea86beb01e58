"""The jet-coiling scene's surface tension on the CPU oracle (the reference's model, restated): at
sigma = 0.07 and r = 1.5 mm the free surface of a resting pool is driven to tens of m/s
within a few steps and the CFL step falls to its minimum; sigma * (r / 25 mm)^3 keeps it
at rest. The jet form of the benchmark therefore runs the scaled coefficient."""
import numpy as np

from oracle import oracle as O
from vfd_gb300 import scenes


def _run(sigma, steps=4):
    s = scenes.jet_coiling_8m(pool=(24, 6, 24))
    s["desc"]["SurfaceTension"] = sigma
    o = O.scene_oracle(s, 32)
    for _ in range(steps):
        st = o.step()
    _, v, _ = o.state()
    return float(np.abs(v).max()), st["TimeStepSize"]


def test_literal_coefficient_drives_the_surface():
    vmax, dt = _run(0.07)
    assert vmax > 10.0 and dt == np.float32(1e-4)


def test_scaled_coefficient_keeps_the_pool_at_rest():
    vmax, dt = _run(0.07 * (0.0015 / 0.025) ** 3)
    assert vmax < 0.5 and dt > 1e-3
