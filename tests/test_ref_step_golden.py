"""The FP32 oracle's step against the reference's own step kernels.

tests/golden/ref_step.npz holds what the reference's DFSPHKernels.cu computes (compiled
for the CPU with a CUDA/glm stand-in, its host loop restated with the oracle's
deterministic reduction rules; tests/golden/make_ref_step.py) over five steps of three
seeded 1,000-particle dam breaks (plain, with the viscosity solve, and with viscosity and
surface tension) and of three benchmark workloads (the 8,000-particle dam break as
configured, the 1M configuration's parameters at 64,000 particles and the 33,401-particle
viscous drop; every 8th or 32nd particle kept). The oracle restates the same kernels, with the GPU's fast-math square
roots and divisions where the reference's CUDA build has them (the CPU build of the
reference rounds those exactly). Tolerances: every solver iteration count and surface-
tension sample count equal; time steps within 1e-3 relative (the adaptive step follows
the fastest particle's |v + a dt|^2: on the 8,000-particle dam break a particle splashing
off the corner, whose speed the square-root roundings move by 6e-4 in the fifth step --
the FP32 and FP64 oracles differ by as much there -- elsewhere by ~1e-5); densities and DFSPH factors
after the first step within 1e-6 relative at the median, 1e-3 at the 99th percentile and
1e-2 at the maximum (a boundary sample's table index can flip with the rounding of a square
root, and a factor's sum of squared gradients then moves most); positions after the first
and the last step within 1e-6 h at the median and 2e-4 h at the maximum; velocities within
1e-4 m/s at the median. The CUDA step is held to the same fixture in
tests/test_gpu_parity.py."""
import os
import sys

import numpy as np
import pytest

from oracle import oracle as O
from vfd_gb300 import _abi

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_ref_step as M  # noqa: E402

GOLDEN = np.load(os.path.join(HERE, "golden", "ref_step.npz"))
ITERS = ("DivergenceSolverIterationCount", "PressureSolverIterationCount", "ViscositySolverIterationCount")


# After the fifth step of the 8,000-particle dam break the time steps differ by 3e-4
# (above), which moves every particle by its speed times that (1.8e-4 h at the median) and
# its velocity by its acceleration times that (3.5e-3 m/s at the median): (position median,
# position maximum in h, velocity median in m/s) for the last step.
LAST_STEP = {"dam_break_8k": (5e-4, 5e-3, 1e-2)}


def check_against_fixture(name, scene, step, state, field=None, pos_median=1e-6, pos_max=2e-4):
    """Runs `step()` M.STEPS times (returning the stats dict) and compares with the
    reference's kernels: state() -> (x, v) after a step, field(kind) -> densities or factors;
    position tolerances in h (the last step's widened for the cases listed above)."""
    g = {k[len(name) + 1:]: GOLDEN[k] for k in GOLDEN.files if k.startswith(name + "/")}
    h = 4 * scene["desc"]["ParticleRadius"]
    sub = M.STRIDE.get(name, 1)  # the fixture keeps every sub-th particle
    for k in range(M.STEPS):
        st = step()
        for key in ITERS:
            assert int(st[key]) == int(g[key][k]), (name, k, key, st[key], g[key][k])
        assert st["TimeStepSize"] == pytest.approx(float(g["TimeStepSize"][k]), rel=1e-3)
        if k == 0 and field is not None:
            for kind, ref in ((_abi.FIELD_DENSITY, g["density1"]), (_abi.FIELD_FACTOR, g["factor1"])):
                rel = np.abs(field(kind)[::sub] - ref) / np.maximum(np.abs(ref), 1e-30)
                assert np.median(rel) < 1e-6 and np.quantile(rel, 0.99) < 1e-3 and rel.max() < 1e-2, \
                    (name, kind, np.median(rel), np.quantile(rel, 0.99), rel.max())
        if k in (0, M.STEPS - 1):
            x, v = state()
            dx = np.abs(np.asarray(x, np.float64)[::sub] - g[f"x{k + 1}"]).max(axis=1) / h
            dv = np.abs(np.asarray(v, np.float64)[::sub] - g[f"v{k + 1}"]).max(axis=1)
            med, mx, vmed = pos_median, pos_max, 1e-4
            if k == M.STEPS - 1 and name in LAST_STEP:
                med, mx, vmed = (max(a, b) for a, b in zip((med, mx, vmed), LAST_STEP[name]))
            assert np.median(dx) < med and dx.max() < mx, (name, k, np.median(dx), dx.max())
            assert np.median(dv) < vmed, (name, k, np.median(dv))


@pytest.mark.parametrize("name", sorted(M.cases()))
def test_oracle_step_equals_reference_kernels(name):
    scene = M.cases()[name]
    o = O.scene_oracle(scene, 32, maps=M.box_maps(scene))

    def state():
        x, v, _ = o.state()
        return x, v

    check_against_fixture(name, scene, o.step, state, o.field)
    if name == "surface_tension":
        assert int(GOLDEN[name + "/SurfaceTensionSampleCount"][-1]) > 0


@pytest.mark.skipif(not os.path.exists(M.LIB), reason="the reference's step kernels are built only where its "
                                                      "sources are (oracle/Makefile target ref)")
@pytest.mark.parametrize("name", ["plain", "viscous"])
def test_reference_step_library_reproduces_the_fixture(name):
    """The committed fixture is what the compiled reference kernels compute: rerun, bit for bit."""
    out = M.run(M.open_lib(), M.cases()[name], M.STRIDE.get(name, 1))
    for key, val in out.items():
        np.testing.assert_array_equal(val, GOLDEN[f"{name}/{key}"], err_msg=key)
