"""ctypes mirrors of the structs in include/vfd_dfsph.h.

The field names are those of the reference's DFSPHSimulationDescription
(Simulation/DFSPH/Structures/DFSPHSimulationDescription.h:9-49),
DFSPHDebugInfo (Structures/DFSPHDebugInfo.h:8-28), DFSPHSimulationInfo
(Structures/DFSPHSimulationInfo.h:5-44) and SDFDeviceData
(Utility/SDF/SDFDeviceData.cuh:549-566).
"""
from __future__ import annotations

import ctypes as C

VFD_OK = 0
VFD_POSITIONS_ABSOLUTE = 0
VFD_POSITIONS_CELL_RELATIVE = 1
VFD_KERNEL_TABLE = 0
VFD_KERNEL_ANALYTIC = 1
VFD_WARM_COLD = 0
VFD_WARM_PREVIOUS = 1
VFD_WARM_EXTRAPOLATE = 2
WARM_COLD, WARM_PREVIOUS, WARM_EXTRAPOLATE = VFD_WARM_COLD, VFD_WARM_PREVIOUS, VFD_WARM_EXTRAPOLATE
VFD_SAMPLE_MIN_DENSITY = 0
VFD_SAMPLE_MEDIUM_DENSITY = 1
VFD_SAMPLE_MAX_DENSITY = 2
VFD_E_ARG = 1
VFD_E_CUDA = 2
VFD_E_NONCONVERGED = 3
VFD_E_NAN = 4
VFD_E_CAPACITY = 5
VFD_E_STATE = 6
VFD_E_NOMEM = 7
VFD_E_NODEVICE = 8

STATUS_NAMES = {
    VFD_OK: "VFD_OK", VFD_E_ARG: "VFD_E_ARG", VFD_E_CUDA: "VFD_E_CUDA",
    VFD_E_NONCONVERGED: "VFD_E_NONCONVERGED", VFD_E_NAN: "VFD_E_NAN",
    VFD_E_CAPACITY: "VFD_E_CAPACITY", VFD_E_STATE: "VFD_E_STATE",
    VFD_E_NOMEM: "VFD_E_NOMEM", VFD_E_NODEVICE: "VFD_E_NODEVICE",
}

FLAG_PRESSURE_CAP = 0x1
FLAG_DIVERGENCE_CAP = 0x2
FLAG_VISCOSITY_CAP = 0x4
FLAG_NEIGHBOR_CAP = 0x8
FLAG_NAN = 0x10
FLAG_GRID_CAPACITY = 0x20

MAX_NEIGHBORS = 70

# Bits of vfd_step_stats.Flags.
VFD_FLAG_PRESSURE_CAP = 0x1
VFD_FLAG_DIVERGENCE_CAP = 0x2
VFD_FLAG_VISCOSITY_CAP = 0x4
VFD_FLAG_NEIGHBOR_CAP = 0x8
VFD_FLAG_NAN = 0x10
VFD_FLAG_GRID_CAPACITY = 0x20
VFD_FLAG_ANCHOR_RANGE = 0x40
VFD_FLAG_BOUNDS = 0x80

FIELD_DENSITY = 0
FIELD_FACTOR = 1
FIELD_DENSITY_ADVECTION = 2
FIELD_PRESSURE_RHO2 = 3
FIELD_PRESSURE_RHO2_V = 4
FIELD_PRESSURE_RESIDUUM = 5
FIELD_PRESSURE_ACCELERATION = 6
FIELD_VELOCITY_DIFFERENCE = 7
FIELD_SURFACE_NORMAL = 8
FIELD_SURFACE_CURVATURE = 9
FIELD_DELTA_FINAL_CURVATURE = 10
FIELD_BOUNDARY_XJ = 11
FIELD_BOUNDARY_VOLUME = 12
FIELD_SURFACE_NORMAL_SMOOTH = 13
FIELD_SURFACE_CURVATURE_SMOOTH = 14

VECTOR_FIELDS = {FIELD_PRESSURE_ACCELERATION, FIELD_VELOCITY_DIFFERENCE, FIELD_SURFACE_NORMAL,
                 FIELD_BOUNDARY_XJ, FIELD_SURFACE_NORMAL_SMOOTH}


class vfd_desc(C.Structure):
    _fields_ = [
        ("TimeStepSize", C.c_float),
        ("MinTimeStepSize", C.c_float),
        ("MaxTimeStepSize", C.c_float),
        ("FrameLength", C.c_float),
        ("FrameCount", C.c_uint32),
        ("MinPressureSolverIterations", C.c_uint32),
        ("MaxPressureSolverIterations", C.c_uint32),
        ("MaxPressureSolverError", C.c_float),
        ("EnableDivergenceSolverError", C.c_int32),
        ("MinDivergenceSolverIterations", C.c_uint32),
        ("MaxDivergenceSolverIterations", C.c_uint32),
        ("MaxDivergenceSolverError", C.c_float),
        ("EnableViscositySolver", C.c_int32),
        ("MinViscositySolverIterations", C.c_uint32),
        ("MaxViscositySolverIterations", C.c_uint32),
        ("MaxViscositySolverError", C.c_float),
        ("Viscosity", C.c_float),
        ("BoundaryViscosity", C.c_float),
        ("TangentialDistanceFactor", C.c_float),
        ("EnableSurfaceTensionSolver", C.c_int32),
        ("SurfaceTensionSmoothPassCount", C.c_uint32),
        ("SurfaceTension", C.c_float),
        ("TemporalSmoothing", C.c_int32),
        ("CSDFix", C.c_int32),
        ("CSD", C.c_int32),
        ("ParticleRadius", C.c_float),
        ("Gravity", C.c_float * 3),
    ]


class vfd_volume_map(C.Structure):
    _fields_ = [
        ("nodes", C.POINTER(C.c_float)),
        ("cells", C.POINTER(C.c_uint32)),
        ("cell_map", C.POINTER(C.c_uint32)),
        ("domain_min", C.c_float * 3),
        ("domain_max", C.c_float * 3),
        ("resolution", C.c_uint32 * 3),
        ("cell_size", C.c_float * 3),
        ("cell_size_inverse", C.c_float * 3),
        ("field_count", C.c_uint32),
        ("node_count", C.c_uint32),
        ("cell_count", C.c_uint32),
        ("cell_map_count", C.c_uint32),
    ]


class vfd_step_stats(C.Structure):
    _fields_ = [
        ("IterationCount", C.c_uint32),
        ("DivergenceSolverIterationCount", C.c_uint32),
        ("PressureSolverIterationCount", C.c_uint32),
        ("ViscositySolverIterationCount", C.c_uint32),
        ("DivergenceSolverError", C.c_float),
        ("PressureSolverError", C.c_float),
        ("ViscositySolverError", C.c_float),
        ("FrameTime", C.c_float),
        ("FrameIndex", C.c_uint32),
        ("TimeStepSize", C.c_float),
        ("MaxVelocityMagnitude", C.c_float),
        ("MaxNeighborCount", C.c_uint32),
        ("Flags", C.c_uint32),
        ("SurfaceTensionSampleCount", C.c_uint32),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class vfd_adjoint_stats(C.Structure):
    _fields_ = [
        ("Steps", C.c_uint32),
        ("ReplayedSteps", C.c_uint32),
        ("ViscositySolves", C.c_uint32),
        ("ViscositySolverIterations", C.c_uint32),
        ("MaxViscositySolverIterations", C.c_uint32),
    ]

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class vfd_info(C.Structure):
    _fields_ = [
        ("ParticleCount", C.c_uint32),
        ("RigidBodyCount", C.c_uint32),
        ("SupportRadius", C.c_float),
        ("SupportRadius2", C.c_float),
        ("ParticleRadius", C.c_float),
        ("ParticleDiameter", C.c_float),
        ("TimeStepSize", C.c_float),
        ("TimeStepSize2", C.c_float),
        ("TimeStepSizeInverse", C.c_float),
        ("TimeStepSize2Inverse", C.c_float),
        ("Volume", C.c_float),
        ("Density0", C.c_float),
        ("ParticleMass", C.c_float),
        ("ParticleMassInverse", C.c_float),
        ("Viscosity", C.c_float),
        ("BoundaryViscosity", C.c_float),
        ("DynamicViscosity", C.c_float),
        ("DynamicBoundaryViscosity", C.c_float),
        ("TangentialDistanceFactor", C.c_float),
        ("TangentialDistance", C.c_float),
        ("SurfaceTension", C.c_float),
        ("SurfaceTensionSampleCount", C.c_uint32),
        ("ClassifierSlope", C.c_float),
        ("ClassifierConstant", C.c_float),
        ("TemporalSmoothing", C.c_int32),
        ("SmoothingFactor", C.c_float),
        ("Factor", C.c_float),
        ("NeighborParticleRadius", C.c_float),
        ("MonteCarloFactor", C.c_float),
        ("Gravity", C.c_float * 3),
    ]

    def as_dict(self) -> dict:
        out = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            out[name] = list(v) if name == "Gravity" else v
        return out


# Reference defaults, DFSPHSimulationDescription.h:11-48.
DEFAULTS = dict(
    TimeStepSize=0.001, MinTimeStepSize=0.0001, MaxTimeStepSize=0.005,
    FrameLength=0.0016, FrameCount=200,
    MinPressureSolverIterations=0, MaxPressureSolverIterations=100, MaxPressureSolverError=10.0,
    EnableDivergenceSolverError=1, MinDivergenceSolverIterations=0, MaxDivergenceSolverIterations=100,
    MaxDivergenceSolverError=10.0,
    EnableViscositySolver=1, MinViscositySolverIterations=0, MaxViscositySolverIterations=100,
    MaxViscositySolverError=0.1, Viscosity=10.0, BoundaryViscosity=10.0, TangentialDistanceFactor=0.5,
    EnableSurfaceTensionSolver=1, SurfaceTensionSmoothPassCount=1, SurfaceTension=1.0,
    TemporalSmoothing=0, CSDFix=-1, CSD=10000,
    ParticleRadius=0.025, Gravity=(0.0, -9.81, 0.0),
)


def make_desc(**overrides) -> vfd_desc:
    """A vfd_desc with the reference defaults, then `overrides` applied."""
    vals = dict(DEFAULTS)
    for k, v in overrides.items():
        if k not in vals:
            raise KeyError(f"unknown description field {k!r}")
        vals[k] = v
    d = vfd_desc()
    for k, v in vals.items():
        if k == "Gravity":
            d.Gravity[:] = [float(x) for x in v]
        else:
            setattr(d, k, v)
    return d


def desc_to_dict(d: vfd_desc) -> dict:
    out = {}
    for name, _ in vfd_desc._fields_:
        v = getattr(d, name)
        out[name] = list(v) if name == "Gravity" else v
    return out
