"""The legacy SPH pipeline on the GPU (vfd_sph_*) against its CPU oracle: the derived
constants, the sort permutation and every step's positions, velocities, densities and
pressures bit for bit (both run the reference's FP32 operations in its order, the GPU
with round-to-nearest intrinsics and no contraction), through many steps; reset and a
description update behave like the reference's."""
import numpy as np
import pytest

from oracle import oracle as O
from vfd_gb300 import meshes, scenes, sph

pytestmark = pytest.mark.gpu


def _block(n=(12, 12, 12), r=0.004, origin=(-0.2, -0.25, -0.2), seed=3):
    return scenes.lattice_block(n, r, origin, 0.05, scenes.SplitMix64(seed))


def _state_equal(g, o):
    for a, b, name in zip(g.GetState(), o.state(), ("x", "v", "rho", "p")):
        np.testing.assert_array_equal(a, b, err_msg=name)


def test_constants_match_oracle():
    d = sph.make_sph_desc()
    x = _block()
    g = sph.SPHSimulation(d, x)
    o = O.SphOracle(d, x)
    assert g.GetParameters() == o.params()


def test_steps_bit_exact():
    d = sph.make_sph_desc()
    x = _block()
    g = sph.SPHSimulation(d, x)
    o = O.SphOracle(d, x)
    for k in range(6):
        g.Steps(1)
        o.steps(1)
        kg, ig = g.GetSort()
        ko, io = o.sort()
        np.testing.assert_array_equal(kg, ko)
        np.testing.assert_array_equal(ig, io)
        _state_equal(g, o)
    g.Steps(100)
    o.steps(100)
    _state_equal(g, o)


def test_on_update_reset_and_description():
    d = sph.make_sph_desc(StepCount=5)
    x = _block(n=(8, 8, 8))
    g = sph.SPHSimulation(d, x)
    g.OnUpdate()
    o = O.SphOracle(d, x)
    o.steps(5)
    _state_equal(g, o)
    g.Reset()
    xr, vr, _, _ = g.GetState()
    np.testing.assert_array_equal(xr, x)
    assert not vr.any()
    d2 = sph.make_sph_desc(StepCount=5, Viscosity=2.0, WorldMin=(-0.4, -0.3, -0.4), WorldMax=(0.4, 0.3, 0.4))
    g.UpdateDescription(d2)
    g.OnUpdate()
    o2 = O.SphOracle(d2, x)
    o2.steps(5)
    _state_equal(g, o2)


def test_sampled_volume_falls_inside_the_world():
    v, t = meshes.icosphere((0.0, 0.0, 0.0), 0.06, 2)
    x = sph.sample_volumes([dict(vertices=v, triangles=t, position=(0.0, 0.1, 0.0), resolution=(12, 12, 12),
                                 sample_mode=2)])
    assert len(x) > 1000
    d = sph.make_sph_desc()
    g = sph.SPHSimulation(d, x)
    g.Steps(300)
    xs, vs, rho, p = g.GetState()
    assert np.all(np.isfinite(xs)) and xs[:, 1].mean() < 0.1 - 0.02
    assert np.all(xs >= np.array(d.WorldMin) + 4 * d.ParticleRadius - 1e-6)
