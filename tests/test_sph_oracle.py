"""The legacy SPH oracle (oracle/sph_oracle.cpp) on the CPU: its derived constants are
the closed forms of SPHSimulation::UpdateParticles / UpdateGrid, the sort is the stable
(key, index) order, and a block of fluid falls, spreads and stays inside the world box."""
import math

import numpy as np
import pytest

from oracle import oracle as O
from vfd_gb300 import scenes
from vfd_gb300.sph import make_sph_desc


def _block(n=(10, 10, 10), r=0.004, origin=(-0.2, -0.25, -0.2)):
    return scenes.lattice_block(n, r, origin, 0.05, scenes.SplitMix64(3))


def test_constants_are_the_closed_forms():
    d = make_sph_desc()
    o = O.SphOracle(d, _block())
    p = o.params()
    h, r = d.Homogeneity, d.ParticleRadius
    assert p["Poly6Kern"] == pytest.approx(315 / (64 * math.pi * h ** 9), rel=1e-6)
    assert p["SpikyKern"] == pytest.approx(22.5 / (math.pi * h ** 6), rel=1e-6)
    assert p["LapKern"] == pytest.approx(45 / (math.pi * h ** 6), rel=1e-6)
    assert p["ParticleMass"] == pytest.approx(1000 * 4 / 3 * math.pi * r ** 3, rel=1e-6)
    assert p["CellSize"] == pytest.approx(2 * r) and p["GridSize"] == [75, 75, 75]
    assert p["CellCount"] == 75 ** 3 and p["BoundsHardDistance"] == pytest.approx(4 * r)


def test_sort_is_stable_by_key():
    o = O.SphOracle(make_sph_desc(), _block())
    o.steps(1)
    k, i = o.sort()
    assert np.all(np.diff(k.astype(np.int64)) >= 0)
    same = np.diff(k.astype(np.int64)) == 0
    assert np.all(np.diff(i.astype(np.int64))[same] > 0)  # ascending index within a cell
    assert sorted(i.tolist()) == list(range(len(i)))


def test_block_falls_and_stays_inside():
    d = make_sph_desc()
    x0 = _block()
    o = O.SphOracle(d, x0)
    o.steps(200)
    x, v, rho, p = o.state()
    assert np.all(np.isfinite(x)) and np.all(np.isfinite(v))
    lo = np.array(d.WorldMin) + 4 * d.ParticleRadius - 1e-6
    hi = np.array(d.WorldMax) - 4 * d.ParticleRadius + 1e-6
    assert np.all(x >= lo) and np.all(x <= hi)
    assert x[:, 1].mean() < x0[:, 1].mean() - 0.01  # it fell
    assert np.ptp(x[:, 0]) > np.ptp(x0[:, 0])       # and spread
    assert np.median(rho) > 0
