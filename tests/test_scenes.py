"""The synthetic workloads stand in for the benchmark configurations: their sizes,
spacings, jitter, parameters and seeds are those the configurations describe (checked on
the CPU, without a GPU), and they are reproducible from their seeds."""
import numpy as np

from vfd_gb300 import scenes


def _spacing_ok(x, r, jitter_frac):
    # nearest-neighbour distances of a jittered lattice of spacing 2r stay within the jitter
    from scipy.spatial import cKDTree
    d, _ = cKDTree(x.astype(np.float64)).query(x.astype(np.float64), k=2)
    nn = d[:, 1]
    assert nn.min() >= 2 * r * (1 - 2 * jitter_frac) - 1e-7 and nn.max() <= 2 * r * (1 + 2 * jitter_frac) + 1e-7


def test_config1_dam_break():
    s = scenes.dam_break_8k()
    assert len(s["x"]) == 8000 and s["desc"]["ParticleRadius"] == 0.025
    assert s["desc"].get("EnableViscositySolver", 0) == 0 and s["desc"].get("EnableSurfaceTensionSolver", 0) == 0
    _spacing_ok(s["x"], 0.025, 0.05)


def test_config2_viscous_dam_break_small_version():
    s = scenes.viscous_dam_break(n_side=20)  # the 1M scene's parameters at 8k particles
    d = s["desc"]
    assert len(s["x"]) == 8000 and d["ParticleRadius"] == 0.005
    assert abs(d["Viscosity"] * 1000.0 - 50.0) < 1e-9  # 50 Pa s dynamic
    assert d["SurfaceTension"] == 0.05 and d["EnableViscositySolver"] == 1
    _spacing_ok(s["x"], 0.005, 0.05)


def test_config3_uneven_batch():
    batch = scenes.uneven_batch()
    counts = np.array([len(s["x"]) for s in batch])
    mus = np.array([s["desc"]["Viscosity"] * 1000.0 for s in batch])
    assert len(batch) == 256
    assert counts.min() >= 1500 and counts.max() <= 70000 and counts.sum() > 4e6
    assert mus.min() >= 0.01 - 1e-9 and mus.max() <= 100.0 + 1e-9
    assert np.log10(mus).std() > 0.8  # spread log-uniformly over four decades
    again = scenes.uneven_batch()
    assert all(np.array_equal(a["x"], b["x"]) for a, b in zip(batch[:8], again[:8]))


def test_config4_viscous_drop():
    s = scenes.viscous_drop_33k()
    x, v = s["x"].astype(np.float64), s["v"].astype(np.float64)
    assert 30000 < len(x) < 36000 and s["desc"]["Viscosity"] * 1000.0 == 10.0
    c = x.mean(axis=0)
    assert np.linalg.norm(x - c, axis=1).max() <= 0.1 + 0.01  # a sphere of radius 0.1 m
    assert abs(np.linalg.norm(v, axis=1).max() - 0.5) < 1e-6  # Fourier modes scaled to 0.5 m/s
    assert np.array_equal(scenes.viscous_drop_33k()["v"], s["v"])


def test_jet_column_scene_has_pool_and_falling_column():
    s = scenes.jet_column_8m(pool=(20, 5, 20))
    pool = scenes.jet_coiling_8m(pool=(20, 5, 20))
    n0 = len(pool["x"])
    assert len(s["x"]) > n0
    np.testing.assert_array_equal(s["x"][:n0], pool["x"])
    col = s["x"][n0:]
    assert np.all(s["v"][n0:, 1] == -1.0) and np.all(s["v"][:n0] == 0.0)
    assert col[:, 1].max() <= 0.5 + 1e-6 and col[:, 1].min() > pool["x"][:, 1].max()
    far = scenes.jet_column_8m(pool=(20, 5, 20), offset=(1000.0, 0.0, 0.0))
    np.testing.assert_allclose(far["x"][:, 0] - 1000.0, s["x"][:, 0], atol=1e-3)
