"""The analytic kernel mode (vfd_set_kernel_mode): W and gradW from the cubic spline at
|r| instead of the reference's tables. Parity with the FP32 oracle in the same mode (one
step and five steps, the tolerances of the table-mode parity tests), the table mode left
as it was, and the two modes apart by no more than the tables' resolution."""
import numpy as np
import pytest

import vfd_gb300 as V
from oracle import oracle as O
from vfd_gb300 import _abi, scenes

pytestmark = pytest.mark.gpu


def _pair(scene, analytic):
    maps = [V.build_box_map(b["min"], b["max"], b["inverted"], b["padding"], b["resolution"],
                            scene["desc"]["ParticleRadius"]) for b in scene["boxes"]]
    g = V.scene_simulation(scene, maps=maps)
    g.SetKernelMode(analytic)
    g.SetFluidObjects(scene["x"], scene["v"])
    o = O.scene_oracle(scene, 32, maps=[O.VolumeMap.from_arrays(m.nodes, m.cells, m.cell_map, m.meta())
                                        for m in maps])
    o.set_kernel_mode(analytic)
    return g, o


def test_analytic_mode_matches_oracle():
    s = scenes.small_dam_break(n_side=10, viscosity=0.02)
    g, o = _pair(s, True)
    h = 4 * s["desc"]["ParticleRadius"]
    for k in range(5):
        sg, so = g.OnUpdate(), o.step()
        for key in ("PressureSolverIterationCount", "DivergenceSolverIterationCount"):
            assert sg[key] == so[key], (key, sg[key], so[key])
        xg, vg, _ = g.GetState()
        xo, vo, _ = o.state()
        dx = np.abs(xg - xo).max(axis=1)
        assert np.median(dx) < 1e-6 * (k + 1) ** 2 * h and dx.max() < 1e-3 * h, (k, np.median(dx), dx.max())
        if k == 0:
            rho_g, rho_o = g.GetField(_abi.FIELD_DENSITY), o.field(_abi.FIELD_DENSITY)
            rel = np.abs(rho_g / rho_o - 1)
            assert np.median(rel) < 1e-6 and rel.max() < 1e-4


def test_modes_differ_by_the_table_resolution():
    s = scenes.small_dam_break(n_side=10)
    a, _ = _pair(s, True)
    t, _ = _pair(s, False)
    a.OnUpdate()
    t.OnUpdate()
    ra, rt = a.GetField(_abi.FIELD_DENSITY), t.GetField(_abi.FIELD_DENSITY)
    rel = np.abs(ra / rt - 1)
    assert 0 < rel.max() < 1e-3  # a table step is h / 9999
    # back to the table mode: the reference's trajectory again
    t2, _ = _pair(s, False)
    t2.SetKernelMode(True)
    t2.SetKernelMode(False)
    t2.SetFluidObjects(s["x"], s["v"])
    t2.OnUpdate()
    np.testing.assert_array_equal(t2.GetState()[0], t.GetState()[0])
