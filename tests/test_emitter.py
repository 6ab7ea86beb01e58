"""The inflow emitter's host logic with a stand-in simulation (no GPU): the disk lattice,
layers in the disk's plane moving along the inflow, and the layer schedule that keeps
layers one spacing apart whatever the time steps."""
import numpy as np

from vfd_gb300 import emitter


class _Recorder:
    def __init__(self):
        self.calls = []

    def Emit(self, x, v):
        self.calls.append((np.array(x), np.array(v)))


def test_disk_lattice():
    em = emitter.InflowEmitter((0.2, 0.5, 0.2), (0.0, -1.0, 0.0), 0.02, 1.0, 0.005)
    assert len(em.disk) == 13  # points of spacing 1 cm within 2 cm
    assert np.all(np.hypot(em.disk[:, 0], em.disk[:, 1]) <= 0.02 + 1e-12)
    x, v = em.layer()
    assert x.dtype == np.float32 and x.shape == (13, 3)
    np.testing.assert_allclose(x[:, 1], 0.5, atol=1e-7)  # in the disk's plane
    np.testing.assert_allclose(v, np.tile([0.0, -1.0, 0.0], (13, 1)))
    np.testing.assert_allclose(x.mean(axis=0), (0.2, 0.5, 0.2), atol=1e-7)


def test_oblique_direction_keeps_the_disk_orthogonal():
    d = np.array([1.0, -2.0, 0.5])
    em = emitter.InflowEmitter((0.0, 0.0, 0.0), d, 0.03, 2.0, 0.004)
    x, v = em.layer(0.01)
    d /= np.linalg.norm(d)
    np.testing.assert_allclose((x.astype(np.float64) @ d), 0.01, atol=1e-6)
    np.testing.assert_allclose(v.astype(np.float64) @ d, 2.0, rtol=1e-6)


def test_layers_stay_one_spacing_apart():
    # steps of 0.5-12 ms at 1 m/s against a spacing of 1 cm: some steps emit two layers
    em = emitter.InflowEmitter((0.0, 0.0, 0.0), (0.0, 0.0, 1.0), 0.01, 1.0, 0.005)
    sim = _Recorder()
    elapsed, schedule = 0.0, []
    for dt in np.random.default_rng(3).uniform(0.0005, 0.012, 200):
        before = len(sim.calls)
        em.advance(sim, dt)
        elapsed += dt
        schedule += [(elapsed, c[0][0, 2]) for c in sim.calls[before:]]
    assert em.layers == len(sim.calls) == int(np.floor(elapsed / em.spacing + 1e-9))
    assert em.emitted == em.layers * len(em.disk)
    assert any(off >= em.spacing for _, off in schedule)  # a step that emitted two layers
    # advanced to the end at the inflow speed, the layers are one spacing apart
    now = np.array([off + (elapsed - when) * 1.0 for when, off in schedule])
    np.testing.assert_allclose(-np.diff(now), em.spacing, atol=1e-6)
