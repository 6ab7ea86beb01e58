"""The legacy SPH pipeline (vfd_sph_* in include/vfd_sph.h): vfd::SPHSimulation
(Simulation/SPH/SPHSimulation.h:55-142) over the CUDA library, with the reference's
method names. Particle volumes come in as positions (ParticleSampler with the
reference's fixed sampling radius of 3.2 mm, `sample_volumes`)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _check, lib as _lib

_F32P, _U32P = C.POINTER(C.c_float), C.POINTER(C.c_uint32)


class vfd_sph_desc(C.Structure):
    _fields_ = [("ParticleRadius", C.c_float), ("Homogeneity", C.c_float), ("RestDensity", C.c_float),
                ("Stiffness", C.c_float), ("Viscosity", C.c_float), ("TimeStep", C.c_float),
                ("GlobalDamping", C.c_float), ("BoundsStiffness", C.c_float), ("BoundsDamping", C.c_float),
                ("BoundsDampingCritical", C.c_float), ("MaxParticlesInCellCount", C.c_uint32),
                ("StepCount", C.c_uint32), ("Gravity", C.c_float * 3), ("WorldMin", C.c_float * 3),
                ("WorldMax", C.c_float * 3)]


class vfd_sph_params(C.Structure):
    _fields_ = [("SmoothingRadius", C.c_float), ("Poly6Kern", C.c_float), ("SpikyKern", C.c_float),
                ("LapKern", C.c_float), ("ParticleMass", C.c_float), ("MinDens", C.c_float), ("MinDist", C.c_float),
                ("BoundsSoftDistance", C.c_float), ("BoundsHardDistance", C.c_float), ("CellSize", C.c_float),
                ("GridSize", C.c_uint32 * 3), ("CellCount", C.c_uint32), ("ParticleCount", C.c_uint32)]


def make_sph_desc(**kw) -> vfd_sph_desc:
    """A description; fields not given take the values of a small water-like scene."""
    vals = dict(ParticleRadius=0.004, Homogeneity=0.01, RestDensity=1000.0, Stiffness=3.0, Viscosity=0.5,
                TimeStep=0.0016, GlobalDamping=1.0, BoundsStiffness=65536.0, BoundsDamping=0.0,
                BoundsDampingCritical=60.0, MaxParticlesInCellCount=32, StepCount=4, Gravity=(0.0, -9.81, 0.0),
                WorldMin=(-0.3, -0.3, -0.3), WorldMax=(0.3, 0.3, 0.3))
    for k, v in kw.items():
        if k not in vals:
            raise KeyError(f"unknown legacy SPH field {k!r}")
        vals[k] = v
    d = vfd_sph_desc()
    for k, v in vals.items():
        if k in ("Gravity", "WorldMin", "WorldMax"):
            getattr(d, k)[:] = [float(x) for x in v]
        else:
            setattr(d, k, v)
    return d


def _bind():
    L = _lib()
    if getattr(L, "_sph_bound", False):
        return L
    P = C.c_void_p
    sig = {
        "vfd_sph_create": [C.POINTER(vfd_sph_desc), _F32P, C.c_uint32, C.POINTER(P)],
        "vfd_sph_destroy": [P],
        "vfd_sph_on_update": [P],
        "vfd_sph_steps": [P, C.c_uint32],
        "vfd_sph_reset": [P],
        "vfd_sph_update_description": [P, C.POINTER(vfd_sph_desc)],
        "vfd_sph_get_params": [P, C.POINTER(vfd_sph_params)],
        "vfd_sph_get_state": [P, _F32P, _F32P, _F32P, _F32P],
        "vfd_sph_set_velocities": [P, _F32P],
        "vfd_sph_get_sort": [P, _U32P, _U32P],
    }
    for name, args in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = C.c_int if name != "vfd_sph_destroy" else None
    L._sph_bound = True
    return L


def sample_volumes(volumes) -> np.ndarray:
    """SPHSimulation::LoadParticleVolumes (SPHSimulation.cpp:242-254): each volume is a dict
    with vertices, triangles (the mesh, already scaled), position, resolution and sample
    mode; it is sampled with the reference's fixed radius 0.0032 and shifted by position."""
    from . import sample_mesh_volume
    out = []
    for v in volumes:
        x = sample_mesh_volume(v["vertices"], v["triangles"], 0.0032, v.get("resolution", (10, 10, 10)), False,
                               v.get("sample_mode", 0))
        out.append(x + np.asarray(v.get("position", (0.0, 0.0, 0.0)), np.float32))
    return np.concatenate(out).astype(np.float32) if out else np.zeros((0, 3), np.float32)


class SPHSimulation:
    def __init__(self, desc: vfd_sph_desc | dict, positions):
        self._lib = _bind()
        self.desc = desc if isinstance(desc, vfd_sph_desc) else make_sph_desc(**desc)
        x = np.ascontiguousarray(np.asarray(positions, np.float32).reshape(-1, 3))
        self.n = len(x)
        h = C.c_void_p()
        _check(self._lib.vfd_sph_create(C.byref(self.desc), x.ctypes.data_as(_F32P), self.n, C.byref(h)),
               "vfd_sph_create")
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._lib.vfd_sph_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def OnUpdate(self):
        _check(self._lib.vfd_sph_on_update(self._h), "vfd_sph_on_update")

    def Steps(self, count: int):
        _check(self._lib.vfd_sph_steps(self._h, int(count)), "vfd_sph_steps")

    def Reset(self):
        _check(self._lib.vfd_sph_reset(self._h), "vfd_sph_reset")

    def UpdateDescription(self, desc: vfd_sph_desc | dict):
        self.desc = desc if isinstance(desc, vfd_sph_desc) else make_sph_desc(**desc)
        _check(self._lib.vfd_sph_update_description(self._h, C.byref(self.desc)), "vfd_sph_update_description")

    def GetParameters(self) -> dict:
        p = vfd_sph_params()
        _check(self._lib.vfd_sph_get_params(self._h, C.byref(p)), "vfd_sph_get_params")
        return {k: (list(getattr(p, k)) if k == "GridSize" else getattr(p, k)) for k, _ in vfd_sph_params._fields_}

    def GetParticleCount(self) -> int:
        return self.n

    def GetState(self):
        """(positions, velocities, density, pressure) in the caller's order."""
        x = np.zeros((self.n, 3), np.float32)
        v = np.zeros((self.n, 3), np.float32)
        rho = np.zeros(self.n, np.float32)
        p = np.zeros(self.n, np.float32)
        _check(self._lib.vfd_sph_get_state(self._h, x.ctypes.data_as(_F32P), v.ctypes.data_as(_F32P),
                                           rho.ctypes.data_as(_F32P), p.ctypes.data_as(_F32P)), "vfd_sph_get_state")
        return x, v, rho, p

    def SetVelocities(self, v):
        va = np.ascontiguousarray(np.asarray(v, np.float32).reshape(-1, 3))
        if len(va) != self.n:
            raise ValueError("one velocity per particle")
        _check(self._lib.vfd_sph_set_velocities(self._h, va.ctypes.data_as(_F32P)), "vfd_sph_set_velocities")

    def GetSort(self):
        """(cell key, particle index) of every sorted slot of the last step."""
        k = np.zeros(self.n, np.uint32)
        i = np.zeros(self.n, np.uint32)
        _check(self._lib.vfd_sph_get_sort(self._h, k.ctypes.data_as(_U32P), i.ctypes.data_as(_U32P)),
               "vfd_sph_get_sort")
        return k, i
