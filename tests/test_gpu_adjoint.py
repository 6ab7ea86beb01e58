"""The GPU adjoint of the step (vfd_adjoint_forward / vfd_adjoint_backward).

Three checks:
  * against the FP64 CPU reference gradient (oracle/adjoint_ref.py, itself pinned by
    FP64 central differences) on a block falling onto a floor with viscosity, the
    divergence and pressure solves and the CFL step: the full step;
  * against central finite differences of the GPU forward run itself where that run
    is a smooth function of its inputs. The divergence solve drives the velocity
    divergence to zero, which puts its residual clamp min(-rho_adv - f, 0) and the
    pressure clamp max(rho_adv - 1, 0) at their kinks, so FP32 differences with a
    usable step straddle kinks there; those cases are left to the FP64 reference.
  * the same finite differences at 1e-3 with the analytic kernel mode and a fixed time
    step, where the step is smooth: the reference's kernel tables are piecewise constant
    in |r| and the adaptive step follows the fastest particle (an argmax), both kinks
    that finite differences straddle.
The Jacobi iteration counts are pinned (min = max), as finite differences of a solve
that stops at a tolerance jump when the count changes.
"""
import numpy as np
import pytest

import vfd_gb300 as V
from oracle import adjoint_ref as R
from oracle import oracle as O
from vfd_gb300 import scenes

pytestmark = pytest.mark.gpu

R_P = 0.025


def _floor_scene(div: bool, n_side: int = 6, fixed_dt: bool = False):
    rng0 = scenes.SplitMix64(9)
    x0 = scenes.lattice_block((n_side,) * 3, R_P, (0.4, scenes.wall_gap(R_P), 0.4), 0.05, rng0).astype(np.float32)
    desc = dict(ParticleRadius=R_P, Viscosity=0.05, BoundaryViscosity=0.05, EnableViscositySolver=1,
                EnableSurfaceTensionSolver=0, EnableDivergenceSolverError=int(div), MaxViscositySolverError=1e-3,
                MinPressureSolverIterations=3, MaxPressureSolverIterations=3,
                MinDivergenceSolverIterations=2, MaxDivergenceSolverIterations=2, TimeStepSize=0.002,
                MaxTimeStepSize=0.002 if fixed_dt else 0.02, MinTimeStepSize=0.002 if fixed_dt else 0.0001)
    maps = [O.build_box_map((0, 0, 0), (1.0, 1.0, 1.0), True, 0.0, (10, 10, 10), R_P)]
    rng = np.random.default_rng(4)
    v0 = (0.3 * rng.standard_normal(x0.shape) + np.array([0.0, -0.5, 0.0])).astype(np.float32)
    target = x0 + 0.01 * rng.standard_normal(x0.shape)
    return dict(x=x0, v=v0, desc=desc, maps=maps, target=target)


class GpuRun:
    def __init__(self, sc, steps, every, analytic=False):
        self.sc, self.steps, self.every = sc, steps, every
        self.sim = V.DFSPHSimulation(V.make_desc(**sc["desc"]))
        if analytic:
            self.sim.SetKernelMode(True)
        self.sim.SetFluidObjects(sc["x"], sc["v"])
        for m in sc["maps"]:
            self.sim.AddRigidBody(m)

    def start(self, x0, v0, nu, nub):
        d = dict(self.sc["desc"])
        d["Viscosity"], d["BoundaryViscosity"] = nu, nub
        self.sim.SetDescription(d)
        self.sim.SetFluidObjects(x0, v0)

    def loss(self, x0=None, v0=None, nu=None, nub=None):
        d = self.sc["desc"]
        self.start(self.sc["x"] if x0 is None else x0, self.sc["v"] if v0 is None else v0,
                   d["Viscosity"] if nu is None else nu, d["BoundaryViscosity"] if nub is None else nub)
        self.sim.Steps(self.steps)
        x, _, _ = self.sim.GetState()
        return float(np.mean(np.sum((x.astype(np.float64) - self.sc["target"]) ** 2, axis=1)))

    def gradient(self):
        d = self.sc["desc"]
        self.start(self.sc["x"], self.sc["v"], d["Viscosity"], d["BoundaryViscosity"])
        self.sim.AdjointForward(self.steps, self.every)
        x, v, _ = self.sim.GetState()
        xb = (2.0 / len(x)) * (x.astype(np.float64) - self.sc["target"])
        x0b, v0b, pb = self.sim.AdjointBackward(xb.astype(np.float32), np.zeros_like(v))
        x2, v2, _ = self.sim.GetState()
        return dict(x=x, v=v, x_after=x2, v_after=v2, x0b=x0b.astype(np.float64), v0b=v0b.astype(np.float64),
                    pb=pb.astype(np.float64))


def _direction(shape, seed):
    d = np.random.default_rng(seed).standard_normal(shape)
    return d / np.sqrt(np.mean(d * d))


def _check(name, adj, ref, tol):
    rel = abs(adj - ref) / max(abs(ref), 1e-30)
    print(f"{name}: GPU adjoint {adj:.6e}  reference {ref:.6e}  relative error {rel:.2e}")
    assert rel < tol, f"{name}: {adj} vs {ref} (relative error {rel:.3e})"


# ------------------------------------------------------------ FP64 reference, full step
@pytest.fixture(scope="module")
def full():
    sc = _floor_scene(div=True)
    steps = 6
    gpu = GpuRun(sc, steps, 4).gradient()
    roll = R.Rollout(sc["desc"], sc["maps"])
    x, v = roll.forward(sc["x"].astype(np.float64), sc["v"].astype(np.float64), steps)
    x0b, v0b, pb = roll.backward(2.0 / len(x) * (x - sc["target"]), np.zeros_like(v))
    assert all(st.cfl for st in roll.steps) and any(b["valid"].any() for st in roll.steps for b in st.bd)
    return sc, gpu, dict(x=x, x0b=x0b, v0b=v0b, pb=pb)


def test_adjoint_leaves_the_final_state(full):
    _, gpu, _ = full
    np.testing.assert_array_equal(gpu["x"], gpu["x_after"])
    np.testing.assert_array_equal(gpu["v"], gpu["v_after"])


def test_forward_matches_fp64_reference(full):
    _, gpu, ref = full
    err = np.abs(gpu["x"] - ref["x"]).max()
    print(f"max |x_GPU - x_FP64| after 6 steps: {err:.3e} m")
    assert err < 1e-4


def test_adjoint_matches_fp64_reference(full):
    # GPU (table kernel, FP32) and reference (analytic kernel, FP64) trajectories drift
    # apart by ~1e-4 per step, which bounds the agreement of their gradients
    sc, gpu, ref = full
    for key in ("v0b", "x0b"):
        rel = np.linalg.norm(gpu[key] - ref[key]) / np.linalg.norm(ref[key])
        print(f"{key}: relative L2 difference {rel:.2e}")
        assert rel < 5e-3
    _check("dL/dViscosity", gpu["pb"][0], ref["pb"][0], 2e-2)
    _check("dL/dBoundaryViscosity", gpu["pb"][1], ref["pb"][1], 2e-2)


# ------------------------------------------------------------ FP64 reference, full step, like for like
@pytest.fixture(scope="module")
def full_analytic():
    """The full step (divergence and pressure solves, viscosity CG, adaptive CFL step,
    volume-map boundary) with the GPU in analytic kernel mode, the kernel the FP64
    reference evaluates: the two differ by FP32 against FP64 arithmetic only."""
    sc = _floor_scene(div=True)
    steps = 6
    gpu = GpuRun(sc, steps, 4, analytic=True).gradient()
    roll = R.Rollout(sc["desc"], sc["maps"])
    x, v = roll.forward(sc["x"].astype(np.float64), sc["v"].astype(np.float64), steps)
    x0b, v0b, pb = roll.backward(2.0 / len(x) * (x - sc["target"]), np.zeros_like(v))
    return sc, gpu, dict(x=x, x0b=x0b, v0b=v0b, pb=pb)


def test_adjoint_matches_fp64_reference_analytic_kernel(full_analytic):
    """Gradients of the full method within 1e-3 of the FP64 reference (relative L2 for the
    initial positions and velocities, relative for both viscosities)."""
    _, gpu, ref = full_analytic
    assert np.abs(gpu["x"] - ref["x"]).max() < 1e-5
    for key in ("v0b", "x0b"):
        rel = np.linalg.norm(gpu[key] - ref[key]) / np.linalg.norm(ref[key])
        print(f"{key}: relative L2 difference {rel:.2e}")
        assert rel < 1e-3, (key, rel)
    _check("dL/dViscosity (analytic kernel)", gpu["pb"][0], ref["pb"][0], 1e-3)
    _check("dL/dBoundaryViscosity (analytic kernel)", gpu["pb"][1], ref["pb"][1], 1e-3)


def test_adjoint_full_size_drop_matches_fp64_reference():
    """The differentiable configuration at its full size: the 33,401-particle viscous drop
    (10 Pa s; the divergence and pressure solves, the viscosity CG, the adaptive CFL step
    and the volume-map boundary all on), 3 steps, the GPU in analytic kernel mode. The
    gradients with respect to the initial positions and velocities (relative L2) and to
    the viscosity are within 1e-3 of the FP64 reference. The drop stays clear of the
    walls in these steps, so dL/dBoundaryViscosity is zero in both.

    The viscosity solve is differentiated at its solution (implicit function theorem) and
    the reference solves exactly, so the forward CG runs to a relative residual of 1e-6
    (MaxViscositySolverError 1e-3, as in the floor scene above). At the configured 1e-2
    (residual 1e-4) the GPU's forward solution is that much off the exact one, and the
    gradients differ by 4.5e-3 (v0), 2.3e-3 (x0) and 2.6e-4 (viscosity), whatever the
    adjoint solve's own tolerance."""
    s = scenes.viscous_drop_33k()
    s["desc"] = dict(s["desc"], MaxViscositySolverError=1e-3)
    r = s["desc"]["ParticleRadius"]
    maps = [O.build_box_map(b["min"], b["max"], b["inverted"], b["padding"], b["resolution"], r) for b in s["boxes"]]
    rng = np.random.default_rng(scenes.config_seed(4))
    target = s["x"].astype(np.float64) + np.array([0.05, -0.2, 0.0]) + 0.25 * r * rng.standard_normal(s["x"].shape)
    sc = dict(x=s["x"], v=s["v"], desc=s["desc"], maps=maps, target=target)
    steps = 3
    gpu = GpuRun(sc, steps, steps, analytic=True).gradient()
    roll = R.Rollout(s["desc"], maps)
    x, v = roll.forward(s["x"].astype(np.float64), s["v"].astype(np.float64), steps)
    x0b, v0b, pb = roll.backward(2.0 / len(x) * (x - target), np.zeros_like(v))
    assert np.abs(gpu["x"] - x).max() < 1e-5
    for key, ref in (("v0b", v0b), ("x0b", x0b)):
        rel = np.linalg.norm(gpu[key] - ref) / np.linalg.norm(ref)
        print(f"{key}: relative L2 difference {rel:.2e}")
        assert rel < 1e-3, (key, rel)
    _check("dL/dViscosity (33k drop, analytic kernel)", gpu["pb"][0], pb[0], 1e-3)
    assert gpu["pb"][1] == 0.0 and pb[1] == 0.0


def test_warm_start_modes_agree_and_count():
    """The three initial guesses of the adjoint viscosity solves (cold, previous lambda,
    extrapolated) give the same gradients to the solve's tolerance; the counters report
    every step's solve and the replayed segments (the last is recorded in the forward run)."""
    sc = _floor_scene(div=True)
    run = GpuRun(sc, 12, 4, analytic=True)
    out = {}
    for mode in (V._abi.WARM_COLD, V._abi.WARM_PREVIOUS, V._abi.WARM_EXTRAPOLATE):
        run.sim.AdjointSetWarmStart(mode)
        out[mode] = (run.gradient(), run.sim.AdjointStats())
    ref, st0 = out[V._abi.WARM_COLD]
    assert st0["Steps"] == 12 and st0["ReplayedSteps"] == 8 and st0["ViscositySolves"] == 12
    assert 0 < st0["MaxViscositySolverIterations"] <= st0["ViscositySolverIterations"]
    for mode, (g, st) in out.items():
        print(f"warm start {mode}: {st}")
        for key in ("v0b", "x0b"):
            rel = np.linalg.norm(g[key] - ref[key]) / np.linalg.norm(ref[key])
            assert rel < 1e-4, (mode, key, rel)
        assert np.abs(g["pb"] - ref["pb"]).max() <= 1e-4 * np.abs(ref["pb"]).max()
    with pytest.raises(V.VFDError):
        run.sim.AdjointSetWarmStart(3)
    for bad in (0.0, -0.1, 1.5, float("nan")):
        with pytest.raises(V.VFDError):
            run.sim.AdjointSetTolerance(bad)


def test_tighter_adjoint_tolerance_converges_to_the_same_gradient():
    """A tenth of the forward's tolerance changes the gradients by no more than the solves'
    own tolerance allows, and costs iterations."""
    sc = _floor_scene(div=True)
    run = GpuRun(sc, 12, 4, analytic=True)
    g1, st1 = run.gradient(), run.sim.AdjointStats()
    run.sim.AdjointSetTolerance(0.1)
    g2, st2 = run.gradient(), run.sim.AdjointStats()
    assert st2["ViscositySolverIterations"] >= st1["ViscositySolverIterations"]
    for key in ("v0b", "x0b"):
        rel = np.linalg.norm(g1[key] - g2[key]) / np.linalg.norm(g2[key])
        assert rel < 1e-4, (key, rel)


def test_backward_graph_matches_host_launches():
    """The backward pass as one graph per step (device-side loops) and launched kernel by
    kernel from the host (loops counted on the host) run the same kernels: the gradients
    agree to the last bits the FP64 atomics of the parameter sums leave free."""
    sc = _floor_scene(div=True)
    out = []
    for graph in (True, False):
        run = GpuRun(sc, 10, 4)
        run.sim.SetGraphMode(graph)
        out.append(run.gradient())
    g, e = out
    for key in ("v0b", "x0b"):
        np.testing.assert_allclose(g[key], e[key], rtol=1e-5, atol=1e-6 * np.abs(e[key]).max())
    np.testing.assert_allclose(g["pb"], e["pb"], rtol=1e-5)


def test_adjoint_after_the_boundary_changes():
    """Replacing the volume maps releases the recorded run, with the copy of the simulation
    that replays its segments (which borrowed the old maps): a later run on the new maps
    matches a fresh simulation's."""
    sc = _floor_scene(div=True)
    run = GpuRun(sc, 8, 4)
    run.gradient()  # two segments: the replaying copy is made
    moved = O.build_box_map((0, 0, 0), (1.0, 0.9, 1.0), True, 0.0, (10, 10, 10), R_P)
    run.sim.SetRigidBodies([moved])
    g = run.gradient()
    fresh = GpuRun(dict(sc, maps=[moved]), 8, 4).gradient()
    for key in ("x0b", "v0b", "pb"):
        np.testing.assert_allclose(g[key], fresh[key], rtol=1e-5, atol=1e-7 * np.abs(fresh[key]).max())


# ------------------------------------------------------------ finite differences, smooth step
@pytest.fixture(scope="module")
def smooth():
    sc = _floor_scene(div=False)
    run = GpuRun(sc, 6, 4)
    return run, run.gradient()


def test_adjoint_velocity_finite_difference(smooth):
    run, g = smooth
    d = _direction(run.sc["v"].shape, 3)
    eps = 2e-2
    fd = (run.loss(v0=(run.sc["v"] + eps * d).astype(np.float32)) -
          run.loss(v0=(run.sc["v"] - eps * d).astype(np.float32))) / (2 * eps)
    _check("dL/dv0 . d (finite difference)", float(np.sum(g["v0b"] * d)), fd, 5e-2)


def test_adjoint_viscosity_finite_difference(smooth):
    run, g = smooth
    nu, nub = run.sc["desc"]["Viscosity"], run.sc["desc"]["BoundaryViscosity"]
    eps = 1e-2
    fd = (run.loss(nu=nu * (1 + eps), nub=nub * (1 + eps)) - run.loss(nu=nu * (1 - eps), nub=nub * (1 - eps))) / (2 * eps)
    _check("dL/dlog(viscosity) (finite difference)", float(g["pb"][0] * nu + g["pb"][1] * nub), fd, 5e-2)


def test_adjoint_position_finite_difference(smooth):
    run, g = smooth
    d = _direction(run.sc["x"].shape, 4)
    eps = 1e-3
    fd = (run.loss(x0=(run.sc["x"] + eps * d).astype(np.float32)) -
          run.loss(x0=(run.sc["x"] - eps * d).astype(np.float32))) / (2 * eps)
    # the kernel table is piecewise constant in |r|: finite differences of positions see
    # quantised kernel values, so this check is looser than the FP64 one above
    _check("dL/dx0 . d (finite difference)", float(np.sum(g["x0b"] * d)), fd, 1e-1)


# ------------------------------------------------------------ analytic kernel, fixed step
@pytest.fixture(scope="module")
def smooth_analytic():
    sc = _floor_scene(div=False, fixed_dt=True)
    run = GpuRun(sc, 6, 4, analytic=True)
    return run, run.gradient()


@pytest.mark.parametrize("along_gradient", [True, False])
def test_analytic_velocity_finite_difference(smooth_analytic, along_gradient):
    run, g = smooth_analytic
    # along the gradient the loss changes most, far above FP32 rounding; a random
    # direction is nearly orthogonal to it, so its difference carries more rounding
    d = g["v0b"] / np.sqrt(np.mean(g["v0b"] ** 2)) if along_gradient else _direction(run.sc["v"].shape, 3)
    eps = 2e-3
    fd = (run.loss(v0=(run.sc["v"] + eps * d).astype(np.float32)) -
          run.loss(v0=(run.sc["v"] - eps * d).astype(np.float32))) / (2 * eps)
    _check("dL/dv0 . d (analytic kernel, finite difference)", float(np.sum(g["v0b"] * d)), fd,
           1e-3 if along_gradient else 3e-3)


def test_analytic_viscosity_finite_difference(smooth_analytic):
    run, g = smooth_analytic
    nu, nub = run.sc["desc"]["Viscosity"], run.sc["desc"]["BoundaryViscosity"]
    eps = 1e-2  # six fixed steps: the viscosity moves the loss little, so a wider step
    fd = (run.loss(nu=nu * (1 + eps), nub=nub * (1 + eps)) - run.loss(nu=nu * (1 - eps), nub=nub * (1 - eps))) / (2 * eps)
    _check("dL/dlog(viscosity) (analytic kernel, finite difference)", float(g["pb"][0] * nu + g["pb"][1] * nub), fd,
           1e-3)


def test_analytic_position_finite_difference(smooth_analytic):
    run, g = smooth_analytic
    d = _direction(run.sc["x"].shape, 4)
    eps = 1e-4
    fd = (run.loss(x0=(run.sc["x"] + eps * d).astype(np.float32)) -
          run.loss(x0=(run.sc["x"] - eps * d).astype(np.float32))) / (2 * eps)
    # positions also move the boundary samples through the volume map, whose
    # interpolation is only continuous across map cells
    _check("dL/dx0 . d (analytic kernel, finite difference)", float(np.sum(g["x0b"] * d)), fd, 5e-3)


# ------------------------------------------------------------ wrapper and errors
def test_torch_rollout_gradients_match_the_adjoint(smooth):
    torch = pytest.importorskip("torch")
    from vfd_gb300.autograd import rollout
    run, g = smooth
    sc = run.sc
    x0 = torch.tensor(sc["x"], dtype=torch.float32, requires_grad=True)
    v0 = torch.tensor(sc["v"], dtype=torch.float32, requires_grad=True)
    nu = torch.tensor(sc["desc"]["Viscosity"], requires_grad=True)
    nub = torch.tensor(sc["desc"]["BoundaryViscosity"], requires_grad=True)
    x, v = rollout(run.sim, x0, v0, nu, nub, steps=6, checkpoint_every=4)
    loss = ((x.double() - torch.tensor(sc["target"])) ** 2).sum(1).mean()
    loss.backward()
    np.testing.assert_allclose(v0.grad.numpy(), g["v0b"], rtol=1e-5, atol=1e-12)
    np.testing.assert_allclose(x0.grad.numpy(), g["x0b"], rtol=1e-5, atol=1e-12)
    np.testing.assert_allclose(float(nu.grad), g["pb"][0], rtol=1e-5)
    np.testing.assert_allclose(float(nub.grad), g["pb"][1], rtol=1e-5)


def test_adjoint_rejects_unsupported_runs():
    s = scenes.small_dam_break(n_side=4, surface_tension=0.05)
    sim = V.scene_simulation(s)
    with pytest.raises(V.VFDError) as e:
        sim.AdjointForward(2, 1)
    assert e.value.code == V._abi.VFD_E_ARG
    s2 = scenes.small_dam_break(n_side=4)
    sim2 = V.scene_simulation(s2)
    with pytest.raises(V.VFDError) as e:
        sim2.AdjointBackward(np.zeros((64, 3), np.float32), np.zeros((64, 3), np.float32))
    assert e.value.code == V._abi.VFD_E_STATE
