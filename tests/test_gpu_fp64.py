"""The FP64 GPU path (vfd_set_precision(sim, VFD_PRECISION_FP64)) against the FP64 CPU
oracle, through the C-ABI.

Both compute the reference's step in double precision from the same FP32 inputs and the
same volume maps; they differ only in summation order (the GPU's block partials, the
oracle's OpenMP loops) and libm, so their trajectories agree to a few ulp of double
precision per step. Tolerances: equal iteration counts every step; positions within
1e-9 h after 10 steps of a small viscous dam break with surface tension, and after 60
steps of the 33,401-particle viscous drop; the FP32 paths are held to the FP64 GPU path
elsewhere (bench.py's precision form)."""
import numpy as np
import pytest

import vfd_gb300 as V
from oracle import oracle as O
from vfd_gb300 import _abi, scenes

pytestmark = pytest.mark.gpu

ITER_KEYS = ("PressureSolverIterationCount", "DivergenceSolverIterationCount", "ViscositySolverIterationCount")


def pair64(scene):
    r = scene["desc"]["ParticleRadius"]
    gm = [V.build_box_map(b["min"], b["max"], b["inverted"], b["padding"], b["resolution"], r) for b in scene["boxes"]]
    om = [O.VolumeMap.from_arrays(m.nodes, m.cells, m.cell_map, m.meta()) for m in gm]
    g = V.scene_simulation(scene, maps=gm)
    g.SetPrecision(True)
    return g, O.scene_oracle(scene, 64, maps=om)


def run_and_compare(scene, steps, tol_h):
    g, o = pair64(scene)
    for k in range(steps):
        sg, so = g.OnUpdate(), o.step()
        for key in ITER_KEYS:
            assert sg[key] == so[key], (k, key, sg[key], so[key])
        assert sg["TimeStepSize"] == pytest.approx(so["TimeStepSize"], rel=1e-6)
    h = 4 * scene["desc"]["ParticleRadius"]
    xg, vg = g.GetStateF64()
    xo, vo, _ = o.state()
    err = np.abs(xg - xo).max() / h
    assert err < tol_h, err
    assert np.abs(vg - vo).max() < 1e-6
    rho_g, rho_o = g.GetField(_abi.FIELD_DENSITY), o.field(_abi.FIELD_DENSITY)
    np.testing.assert_allclose(rho_g, rho_o, rtol=1e-6)
    return g


def test_fp64_path_matches_fp64_oracle_small_dam_break():
    s = scenes.small_dam_break(n_side=10, viscosity=0.02, surface_tension=0.05)
    run_and_compare(s, 10, 1e-9)


def test_fp64_path_matches_fp64_oracle_viscous_drop():
    run_and_compare(scenes.viscous_drop_33k(), 60, 1e-9)


def test_fp64_path_refuses_fp32_only_calls_and_switches_back():
    s = scenes.small_dam_break(n_side=6)
    g = V.scene_simulation(s)
    g.SetPrecision(True)
    g.Steps(2)
    x, v, _ = g.GetState()
    with pytest.raises(V.VFDError) as e:
        g.SetState(x, v)
    assert e.value.code == _abi.VFD_E_STATE
    with pytest.raises(V.VFDError) as e:
        g.Checkpoint()
    assert e.value.code == _abi.VFD_E_STATE
    g.SetPrecision(False)  # back to the FP32 step, restarted from the fluid objects
    g.Steps(2)
    with pytest.raises(V.VFDError) as e:
        g.GetStateF64()
    assert e.value.code == _abi.VFD_E_STATE
    assert np.isfinite(g.GetState()[0]).all()
