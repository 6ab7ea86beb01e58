"""Golden steps from the reference's own step kernels.

Builds oracle/_ref/libvfd_refstep.so (the reference's Simulation/DFSPH/DFSPHKernels.cu and
its search kernels compiled for the CPU with a CUDA/glm stand-in header, beside a
restatement of their host loop, oracle/ref_step/driver.cpp; recipe in oracle/Makefile,
target `ref`) and runs it for five steps on three seeded 1,000-particle dam breaks -- plain, with the
viscosity solve, and with viscosity and surface tension -- and on three benchmark
workloads, the 8,000-particle dam break, the 1M configuration's parameters at 64,000
particles and the 33,401-particle viscous drop,
with the volume maps of the oracle's box-map builder. Writes tests/golden/ref_step.npz:
per case and step the solver iteration counts, errors and time step, the densities and
DFSPH factors after the first step, and the positions and velocities after the first and
the last step (of every 8th or 32nd particle in the three larger cases).

Usage: python tests/golden/make_ref_step.py VFD_ROOT
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from vfd_gb300 import _abi, scenes  # noqa: E402

LIB = os.path.join(ROOT, "oracle", "_ref", "libvfd_refstep.so")
OUT = os.path.join(HERE, "ref_step.npz")
STEPS = 5
STATS = ("DivergenceSolverIterationCount", "PressureSolverIterationCount", "ViscositySolverIterationCount",
         "DivergenceSolverError", "PressureSolverError", "ViscositySolverError", "TimeStepSize",
         "MaxVelocityMagnitude", "SurfaceTensionSampleCount")


def cases() -> dict:
    """The seeded scenes, rebuilt identically by the tests."""
    return {
        "plain": scenes.small_dam_break(n_side=10),
        "viscous": scenes.small_dam_break(n_side=10, viscosity=0.05),
        "surface_tension": scenes.small_dam_break(n_side=10, viscosity=0.01, surface_tension=0.05),
        # two benchmark workloads: the 8,000-particle dam break as configured, and the 1M
        # configuration's parameters (viscosity, surface tension, CSD) at 40^3 particles
        "dam_break_8k": scenes.dam_break_8k(),
        "viscous_dam_break_64k": scenes.viscous_dam_break(n_side=40),
        # the differentiable workload: the 33,401-particle viscous drop
        "viscous_drop_33k": scenes.viscous_drop_33k(),
    }


# Every STRIDE-th particle's positions and velocities are kept for the larger cases.
STRIDE = {"dam_break_8k": 8, "viscous_dam_break_64k": 32, "viscous_drop_33k": 32}


def box_maps(scene) -> list:
    r = scene["desc"]["ParticleRadius"]
    return [O.build_box_map(b["min"], b["max"], b["inverted"], b["padding"], b["resolution"], r)
            for b in scene["boxes"]]


def load(vfd_root: str):
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF={vfd_root}"], check=True)
    return open_lib()


def open_lib():
    """The built reference-step library (oracle/_ref/libvfd_refstep.so) with its signatures."""
    lib = C.CDLL(LIB)
    lib.ref_step_create.restype = C.c_void_p
    lib.ref_step_create.argtypes = [C.POINTER(_abi.vfd_desc)]
    lib.ref_step_destroy.argtypes = [C.c_void_p]
    lib.ref_step_add_rigid_body.argtypes = [C.c_void_p, C.POINTER(_abi.vfd_volume_map)]
    lib.ref_step_set_fluid.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32]
    lib.ref_step_step.argtypes = [C.c_void_p, C.POINTER(_abi.vfd_step_stats)]
    lib.ref_step_get_state.argtypes = [C.c_void_p] + [C.c_void_p] * 5
    return lib


def run(lib, scene, stride: int = 1) -> dict:
    maps = box_maps(scene)
    desc = _abi.make_desc(**scene["desc"])
    h = lib.ref_step_create(C.byref(desc))
    for m in maps:
        assert lib.ref_step_add_rigid_body(h, C.byref(m.struct)) == 0
    x0 = np.ascontiguousarray(scene["x"], np.float32)
    v0 = np.ascontiguousarray(scene["v"], np.float32)
    n = len(x0)
    assert lib.ref_step_set_fluid(h, x0.ctypes.data, v0.ctypes.data, n) == 0
    out = {k: [] for k in STATS}
    for k in range(STEPS):
        st = _abi.vfd_step_stats()
        assert lib.ref_step_step(h, C.byref(st)) == 0
        for key in STATS:
            out[key].append(getattr(st, key))
        if k in (0, STEPS - 1):
            x, v = np.zeros((n, 3), np.float32), np.zeros((n, 3), np.float32)
            rho, fac = np.zeros(n, np.float32), np.zeros(n, np.float32)
            lib.ref_step_get_state(h, x.ctypes.data, v.ctypes.data, None, rho.ctypes.data, fac.ctypes.data)
            out[f"x{k + 1}"], out[f"v{k + 1}"] = x[::stride], v[::stride]
            if k == 0:
                out["density1"], out["factor1"] = rho[::stride], fac[::stride]
    lib.ref_step_destroy(h)
    return {k: np.asarray(v) for k, v in out.items()}


def main():
    if len(sys.argv) != 2:
        sys.exit(__doc__)
    lib = load(sys.argv[1])
    arrays = {}
    for name, scene in cases().items():
        for key, val in run(lib, scene, STRIDE.get(name, 1)).items():
            arrays[f"{name}/{key}"] = val
    np.savez_compressed(OUT, **arrays)
    print(f"wrote {OUT} ({os.path.getsize(OUT)} bytes)")


if __name__ == "__main__":
    main()
