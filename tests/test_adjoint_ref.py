"""The FP64 CPU reference gradient (oracle/adjoint_ref.py) against FP64 central
differences of its own forward run: a 125-particle block resting on the floor of a
large box (planar wall contact), with viscosity, the divergence and pressure solves
(fixed iteration counts) and the CFL time step, over three steps."""
import numpy as np
import pytest

from oracle import adjoint_ref as R
from oracle import oracle as O
from vfd_gb300 import scenes


@pytest.fixture(scope="module")
def problem():
    r = 0.025
    rng0 = scenes.SplitMix64(9)
    x0 = scenes.lattice_block((5, 5, 5), r, (0.4, scenes.wall_gap(r), 0.4), 0.05, rng0).astype(np.float64)
    desc = dict(ParticleRadius=r, Viscosity=0.05, BoundaryViscosity=0.05, EnableViscositySolver=1,
                EnableSurfaceTensionSolver=0, EnableDivergenceSolverError=1,
                MinPressureSolverIterations=3, MaxPressureSolverIterations=3,
                MinDivergenceSolverIterations=2, MaxDivergenceSolverIterations=2, TimeStepSize=0.002,
                MaxTimeStepSize=0.05)
    maps = [O.build_box_map((0, 0, 0), (1.0, 1.0, 1.0), True, 0.0, (10, 10, 10), r)]
    rng = np.random.default_rng(4)
    v0 = 0.3 * rng.standard_normal(x0.shape) + np.array([0.0, -0.5, 0.0])
    target = x0 + 0.01 * rng.standard_normal(x0.shape)
    roll = R.Rollout(desc, maps)
    x, v = roll.forward(x0, v0, 3)
    xb = 2.0 / len(x) * (x - target)
    x0b, v0b, pb = roll.backward(xb, np.zeros_like(v))
    return dict(desc=desc, maps=maps, x0=x0, v0=v0, target=target, x0b=x0b, v0b=v0b, pb=pb, roll=roll)


def _loss(p, x0=None, v0=None, desc=None):
    return R.rollout_loss(desc or p["desc"], p["maps"], p["x0"] if x0 is None else x0,
                          p["v0"] if v0 is None else v0, 3, p["target"])


def _rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


def test_reference_scene_is_differentiable(problem):
    st = problem["roll"].steps
    assert all(s.cfl for s in st), "the CFL step should be active"
    assert any(b["valid"].any() for s in st for b in s.bd), "the block should touch the floor"
    assert all(len(s.rd) == 2 and len(s.rp) == 3 for s in st)


def test_reference_velocity_gradient(problem):
    d = np.random.default_rng(1).standard_normal(problem["v0"].shape)
    eps = 1e-6
    fd = (_loss(problem, v0=problem["v0"] + eps * d) - _loss(problem, v0=problem["v0"] - eps * d)) / (2 * eps)
    assert _rel(float(np.sum(problem["v0b"] * d)), fd) < 1e-5


def test_reference_position_gradient(problem):
    d = np.random.default_rng(2).standard_normal(problem["x0"].shape)
    eps = 1e-8
    fd = (_loss(problem, x0=problem["x0"] + eps * d) - _loss(problem, x0=problem["x0"] - eps * d)) / (2 * eps)
    assert _rel(float(np.sum(problem["x0b"] * d)), fd) < 1e-5


@pytest.mark.parametrize("k,name", [(0, "Viscosity"), (1, "BoundaryViscosity")])
def test_reference_viscosity_gradient(problem, k, name):
    nu = problem["desc"][name]
    eps = 1e-6 * nu
    lo, hi = dict(problem["desc"]), dict(problem["desc"])
    lo[name], hi[name] = nu - eps, nu + eps
    fd = (_loss(problem, desc=hi) - _loss(problem, desc=lo)) / (2 * eps)
    assert _rel(float(problem["pb"][k]), fd) < 1e-5


def test_large_scene_paths_match_the_exact_ones(problem, monkeypatch):
    """The k-d tree pair search gives the all-pairs search's pairs in the same order, and
    the CG solve of the viscosity system the direct solve's solution (to 1e-10), on the
    scene above with the size thresholds lowered so both paths run."""
    rng = np.random.default_rng(11)
    x = rng.random((1500, 3)) * 0.4
    h = 0.05
    exact = R._pairs(x, h)
    monkeypatch.setattr(R, "_ALL_PAIRS_MAX", 100)
    tree = R._pairs(x, h)
    for a, b in zip(exact, tree):
        np.testing.assert_array_equal(a, b)
    step = problem["roll"].steps[-1]
    A = step._visc_matrix(step.dto)
    b = rng.standard_normal(A.shape[0])
    direct = R._solve_spd(A, b)
    monkeypatch.setattr(R, "_DIRECT_MAX", 10)
    cg = R._solve_spd(A, b)
    assert np.linalg.norm(cg - direct) <= 1e-10 * np.linalg.norm(direct)
