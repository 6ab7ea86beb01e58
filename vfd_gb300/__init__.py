"""vfd_gb300: a GB300-native DFSPH simulation step behind VFD's solver API.

The compute path is the CUDA library libvfd_dfsph.so (include/vfd_dfsph.h),
loaded through ctypes. This module mirrors the reference's
vfd::DFSPHSimulation (Simulation/DFSPH/DFSPHSimulator.h:10-58): same method
names, same argument meaning; errors raise VFDError instead of exiting the
process. There is no CPU fallback: without the library or a GPU, calls fail.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

from . import _abi
from ._abi import make_desc, vfd_desc, vfd_info, vfd_step_stats, vfd_volume_map  # noqa: F401

HERE = os.path.dirname(os.path.abspath(__file__))
# VFD_LIBRARY selects another build of the library (the bounds-checked variant,
# libvfd_dfsph_checked.so); the default is the in-tree release build.
LIB_PATH = os.environ.get("VFD_LIBRARY") or os.path.join(HERE, "libvfd_dfsph.so")

# Every entry point declared in include/vfd_dfsph.h.
EXPORTS = [
    "vfd_desc_default", "vfd_create", "vfd_destroy", "vfd_set_description", "vfd_get_description",
    "vfd_set_fluid", "vfd_add_rigid_body", "vfd_clear_rigid_bodies", "vfd_box_map_sizes", "vfd_build_box_map",
    "vfd_reset", "vfd_step", "vfd_steps", "vfd_steps_async", "vfd_synchronize", "vfd_simulate",
    "vfd_get_state", "vfd_set_state", "vfd_get_field", "vfd_find_neighbors", "vfd_get_neighbors",
    "vfd_get_info", "vfd_get_particle_count", "vfd_get_current_time_step_size", "vfd_get_max_velocity_magnitude",
    "vfd_get_debug_info", "vfd_get_kernel_table", "vfd_set_graph_mode", "vfd_create_batch",
    "vfd_get_scene_count", "vfd_scene_set_fluid", "vfd_scene_add_rigid_body", "vfd_scene_get_state",
    "vfd_scene_get_stats", "vfd_set_device", "vfd_last_error", "vfd_abi_version", "vfd_profile_kernels",
    "vfd_get_stream", "vfd_get_launch_count", "vfd_set_lanes", "vfd_get_lanes", "vfd_autotune",
    "vfd_find_neighbors_noalloc", "vfd_adjoint_forward", "vfd_adjoint_backward", "vfd_adjoint_release",
    "vfd_set_position_mode", "vfd_build_mesh_map", "vfd_sample_mesh_volume", "vfd_set_kernel_mode",
    "vfd_emit", "vfd_get_graph_mode", "vfd_checkpoint_size", "vfd_checkpoint", "vfd_restore",
    "vfd_set_tiles", "vfd_get_tiles", "vfd_set_precision", "vfd_get_state_f64", "vfd_set_blocks", "vfd_get_blocks",
    "vfd_adjoint_set_warm_start", "vfd_adjoint_get_stats", "vfd_adjoint_set_tolerance",
    # include/vfd_sph.h: the legacy SPH pipeline (vfd_gb300.sph)
    "vfd_sph_create", "vfd_sph_destroy", "vfd_sph_on_update", "vfd_sph_steps", "vfd_sph_reset",
    "vfd_sph_update_description", "vfd_sph_get_params", "vfd_sph_get_state", "vfd_sph_set_velocities",
    "vfd_sph_get_sort",
]

TUNED_KERNELS = ["density_factor", "pressure_accel", "jacobi_iter", "div_finish", "st_classify",
                 "st_smooth", "visc_precond", "visc_setup", "cg_spmv", "pres_init", "pres_finish"]
# the solver-loop passes that run on cell tiles (vfd_set_tiles)
TILE_KERNELS = ["pressure_accel", "jacobi_iter", "cg_spmv"]


class vfd_kernel_time(C.Structure):
    _fields_ = [("name", C.c_char * 48), ("launches", C.c_uint32), ("total_ms", C.c_double)]


class VFDError(RuntimeError):
    def __init__(self, code: int, where: str, message: str):
        self.code = code
        super().__init__(f"{where} -> {_abi.STATUS_NAMES.get(code, code)}: {message}")


_lock = threading.Lock()
_lib = None

FRAME_CALLBACK = C.CFUNCTYPE(None, C.c_uint32, C.c_uint32, C.POINTER(C.c_float), C.POINTER(C.c_float),
                             C.POINTER(C.c_float), C.c_float, C.c_float, C.c_void_p)


def lib() -> C.CDLL:
    """The loaded CUDA library; raises if it was not built."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise ImportError(f"{LIB_PATH} is missing: build it with `python -m vfd_gb300.build` "
                                  "(the DFSPH step has no CPU implementation)")
            L = C.CDLL(LIB_PATH)
            P = C.c_void_p
            u32p, f32p = C.POINTER(C.c_uint32), C.POINTER(C.c_float)
            sig = {
                "vfd_desc_default": [C.POINTER(vfd_desc)],
                "vfd_create": [C.POINTER(vfd_desc), C.POINTER(P)],
                "vfd_destroy": [P],
                "vfd_set_description": [P, C.POINTER(vfd_desc)],
                "vfd_get_description": [P, C.POINTER(vfd_desc)],
                "vfd_set_fluid": [P, f32p, f32p, C.c_uint32],
                "vfd_add_rigid_body": [P, C.POINTER(vfd_volume_map)],
                "vfd_clear_rigid_bodies": [P],
                "vfd_box_map_sizes": [u32p, u32p, u32p],
                "vfd_build_box_map": [f32p, f32p, C.c_int32, C.c_float, u32p, C.c_float, f32p, u32p, u32p,
                                      C.POINTER(vfd_volume_map)],
                "vfd_reset": [P],
                "vfd_step": [P, C.POINTER(vfd_step_stats)],
                "vfd_steps": [P, C.c_uint32, C.POINTER(vfd_step_stats)],
                "vfd_steps_async": [P, C.c_uint32],
                "vfd_synchronize": [P, C.POINTER(vfd_step_stats)],
                "vfd_simulate": [P, FRAME_CALLBACK, C.c_void_p],
                "vfd_get_state": [P, f32p, f32p, f32p],
                "vfd_set_state": [P, f32p, f32p],
                "vfd_get_field": [P, C.c_int32, C.c_uint32, f32p],
                "vfd_find_neighbors": [P],
                "vfd_get_neighbors": [P, u32p, u32p, u32p, C.c_uint32, u32p, u32p, u32p],
                "vfd_get_info": [P, C.POINTER(vfd_info)],
                "vfd_get_particle_count": [P, u32p],
                "vfd_get_current_time_step_size": [P, f32p],
                "vfd_get_max_velocity_magnitude": [P, f32p],
                "vfd_get_debug_info": [P, C.POINTER(vfd_step_stats)],
                "vfd_get_kernel_table": [P, f32p, f32p, f32p, f32p],
                "vfd_set_graph_mode": [P, C.c_int32],
                "vfd_create_batch": [C.POINTER(vfd_desc), C.c_uint32, C.POINTER(P)],
                "vfd_get_scene_count": [P, u32p],
                "vfd_scene_set_fluid": [P, C.c_uint32, f32p, f32p, C.c_uint32],
                "vfd_scene_add_rigid_body": [P, C.c_uint32, C.POINTER(vfd_volume_map)],
                "vfd_scene_get_state": [P, C.c_uint32, f32p, f32p, f32p],
                "vfd_scene_get_stats": [P, C.c_uint32, C.POINTER(vfd_step_stats)],
                "vfd_set_device": [C.c_int32],
                "vfd_profile_kernels": [P, C.c_uint32, C.POINTER(vfd_kernel_time), C.c_uint32, u32p],
                "vfd_get_stream": [P, C.POINTER(C.c_void_p)],
                "vfd_get_launch_count": [P, C.POINTER(C.c_uint64), C.c_int32],
                "vfd_set_lanes": [P, C.POINTER(C.c_uint8), C.c_uint32],
                "vfd_get_lanes": [P, C.POINTER(C.c_uint8), C.c_uint32],
                "vfd_set_tiles": [P, C.POINTER(C.c_uint8), C.c_uint32],
                "vfd_set_precision": [P, C.c_int32],
                "vfd_set_blocks": [P, C.POINTER(C.c_uint16), C.c_uint32],
                "vfd_get_blocks": [P, C.POINTER(C.c_uint16), C.c_uint32],
                "vfd_get_state_f64": [P, C.POINTER(C.c_double), C.POINTER(C.c_double)],
                "vfd_get_tiles": [P, C.POINTER(C.c_uint8), C.c_uint32],
                "vfd_autotune": [P, C.c_uint32, C.POINTER(C.c_uint8), C.c_uint32],
                "vfd_find_neighbors_noalloc": [C.c_void_p, C.c_uint32, C.c_float, C.c_void_p, C.c_void_p,
                                               C.c_void_p, C.c_void_p],
                "vfd_adjoint_forward": [P, C.c_uint32, C.c_uint32, C.POINTER(vfd_step_stats)],
                "vfd_adjoint_backward": [P, f32p, f32p, f32p, f32p, f32p],
                "vfd_adjoint_release": [P],
                "vfd_adjoint_set_warm_start": [P, C.c_int32],
                "vfd_adjoint_set_tolerance": [P, C.c_float],
                "vfd_adjoint_get_stats": [P, C.POINTER(_abi.vfd_adjoint_stats)],
                "vfd_set_position_mode": [P, C.c_int32],
                "vfd_set_kernel_mode": [P, C.c_int32],
                "vfd_emit": [P, f32p, f32p, C.c_uint32],
                "vfd_get_graph_mode": [P, C.POINTER(C.c_int32), C.POINTER(C.c_int32)],
                "vfd_checkpoint_size": [P, C.POINTER(C.c_uint64)],
                "vfd_checkpoint": [P, C.c_void_p, C.c_uint64],
                "vfd_restore": [P, C.c_void_p, C.c_uint64],
                "vfd_build_mesh_map": [f32p, C.c_uint32, u32p, C.c_uint32, f32p, C.c_int32, C.c_float, u32p,
                                       C.c_float, f32p, u32p, u32p, C.POINTER(vfd_volume_map)],
                "vfd_sample_mesh_volume": [f32p, C.c_uint32, u32p, C.c_uint32, f32p, C.c_float, u32p, C.c_int32,
                                           C.c_int32, f32p, C.c_uint32, u32p],
                "vfd_last_error": [],
                "vfd_abi_version": [],
            }
            for name, args in sig.items():
                fn = getattr(L, name)
                fn.argtypes = args
                fn.restype = C.c_int
            L.vfd_last_error.restype = C.c_char_p
            _lib = L
    return _lib


def _check(rc: int, where: str):
    if rc != _abi.VFD_OK:
        msg = lib().vfd_last_error()
        raise VFDError(rc, where, msg.decode() if msg else "")


def _f32(a):
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a, a.ctypes.data_as(C.POINTER(C.c_float))


def _u32ptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint32)) if a is not None else None


def _fptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_float)) if a is not None else None


class VolumeMap:
    """A rigid body's volume map (SDFDeviceData layout) with its arrays kept alive."""

    def __init__(self, nodes, cells, cell_map, struct: vfd_volume_map):
        self.nodes, self.cells, self.cell_map, self.struct = nodes, cells, cell_map, struct

    @staticmethod
    def from_arrays(nodes, cells, cell_map, meta: dict) -> "VolumeMap":
        nodes = np.ascontiguousarray(nodes, np.float32)
        cells = np.ascontiguousarray(cells, np.uint32)
        cell_map = np.ascontiguousarray(cell_map, np.uint32)
        m = vfd_volume_map()
        m.nodes = _fptr(nodes)
        m.cells = _u32ptr(cells)
        m.cell_map = _u32ptr(cell_map)
        for k in ("domain_min", "domain_max", "resolution", "cell_size", "cell_size_inverse"):
            getattr(m, k)[:] = list(meta[k])
        for k in ("field_count", "node_count", "cell_count", "cell_map_count"):
            setattr(m, k, int(meta[k]))
        return VolumeMap(nodes, cells, cell_map, m)

    def meta(self) -> dict:
        m = self.struct
        return dict(domain_min=list(m.domain_min), domain_max=list(m.domain_max), resolution=list(m.resolution),
                    cell_size=list(m.cell_size), cell_size_inverse=list(m.cell_size_inverse),
                    field_count=m.field_count, node_count=m.node_count, cell_count=m.cell_count,
                    cell_map_count=m.cell_map_count)


def build_box_map(bmin, bmax, inverted: bool, padding: float, resolution, particle_radius: float) -> VolumeMap:
    """Volume map of an axis-aligned box, built on the GPU (RigidBody::RigidBody for a box mesh)."""
    res = np.ascontiguousarray(resolution, np.uint32)
    nn, nc = C.c_uint32(), C.c_uint32()
    _check(lib().vfd_box_map_sizes(_u32ptr(res), C.byref(nn), C.byref(nc)), "vfd_box_map_sizes")
    nodes = np.zeros(2 * nn.value, np.float32)
    cells = np.zeros(2 * nc.value * 32, np.uint32)
    cell_map = np.zeros(2 * nc.value, np.uint32)
    m = vfd_volume_map()
    lo, lop = _f32(bmin)
    hi, hip = _f32(bmax)
    _check(lib().vfd_build_box_map(lop, hip, int(bool(inverted)), C.c_float(padding), _u32ptr(res),
                                   C.c_float(particle_radius), _fptr(nodes), _u32ptr(cells), _u32ptr(cell_map),
                                   C.byref(m)), "vfd_build_box_map")
    return VolumeMap(nodes, cells, cell_map, m)


def _mesh_args(vertices, triangles, transform):
    v = np.ascontiguousarray(np.asarray(vertices, np.float32).reshape(-1, 3))
    t = np.ascontiguousarray(np.asarray(triangles, np.uint32).reshape(-1, 3))
    if transform is None:
        return v, t, None, None
    m = np.asarray(transform, np.float32).reshape(4, 4)
    col = np.ascontiguousarray(m.T.reshape(16))  # column-major, as glm stores a mat4
    return v, t, col, _fptr(col)


def build_mesh_map(vertices, triangles, transform=None, inverted: bool = False, padding: float = 0.0,
                   resolution=(20, 20, 20), particle_radius: float = 0.025) -> VolumeMap:
    """Volume map of a closed triangle mesh built on the GPU (RigidBody::RigidBody,
    RigidBody.cu:10-72). `transform` is the body's 4x4 placement matrix (acting on column
    vectors, translation in the last column) or None."""
    res = np.ascontiguousarray(resolution, np.uint32)
    nn, nc = C.c_uint32(), C.c_uint32()
    _check(lib().vfd_box_map_sizes(_u32ptr(res), C.byref(nn), C.byref(nc)), "vfd_box_map_sizes")
    v, t, col, colp = _mesh_args(vertices, triangles, transform)
    nodes = np.zeros(2 * nn.value, np.float32)
    cells = np.zeros(2 * nc.value * 32, np.uint32)
    cell_map = np.zeros(2 * nc.value, np.uint32)
    m = vfd_volume_map()
    _check(lib().vfd_build_mesh_map(_fptr(v), len(v), _u32ptr(t), len(t), colp, int(bool(inverted)),
                                    C.c_float(padding), _u32ptr(res), C.c_float(particle_radius), _fptr(nodes),
                                    _u32ptr(cells), _u32ptr(cell_map), C.byref(m)), "vfd_build_mesh_map")
    return VolumeMap(nodes, cells, cell_map, m)


SAMPLE_MODES = {"min": _abi.VFD_SAMPLE_MIN_DENSITY, "medium": _abi.VFD_SAMPLE_MEDIUM_DENSITY,
                "max": _abi.VFD_SAMPLE_MAX_DENSITY}


def sample_mesh_volume(vertices, triangles, particle_radius: float, resolution=(20, 20, 20), inverted: bool = False,
                       sample_mode=0, transform=None) -> np.ndarray:
    """Particles filling a mesh (ParticleSampler::SampleMeshVolume, ParticleSampler.cpp:7-91,
    on the GPU): an (n, 3) float32 array in the reference's lattice order. `sample_mode` is
    0/1/2 or "min"/"medium"/"max"."""
    mode = SAMPLE_MODES[sample_mode] if isinstance(sample_mode, str) else int(sample_mode)
    res = np.ascontiguousarray(resolution, np.uint32)
    v, t, col, colp = _mesh_args(vertices, triangles, transform)
    count = C.c_uint32()
    args = (_fptr(v), len(v), _u32ptr(t), len(t), colp, C.c_float(particle_radius), _u32ptr(res),
            int(bool(inverted)), mode)
    _check(lib().vfd_sample_mesh_volume(*args, None, 0, C.byref(count)), "vfd_sample_mesh_volume")
    out = np.zeros((count.value, 3), np.float32)
    if count.value:
        _check(lib().vfd_sample_mesh_volume(*args, _fptr(out), count.value, C.byref(count)),
               "vfd_sample_mesh_volume")
    return out


class DFSPHSimulation:
    """vfd::DFSPHSimulation (DFSPHSimulator.h:10-58) over the CUDA library.

    One instance holds one device simulation. `scenes` > 1 creates a batch of
    independent scenes advanced together (scene-scoped methods take `scene=`).
    """

    def __init__(self, desc: vfd_desc | dict | None = None, scenes: list | None = None):
        if scenes is not None:
            descs = [d if isinstance(d, vfd_desc) else make_desc(**d) for d in scenes]
        else:
            if desc is None:
                desc = vfd_desc()
                _check(lib().vfd_desc_default(C.byref(desc)), "vfd_desc_default")
            descs = [desc if isinstance(desc, vfd_desc) else make_desc(**desc)]
        arr = (vfd_desc * len(descs))(*descs)
        h = C.c_void_p()
        _check(lib().vfd_create_batch(arr, len(descs), C.byref(h)), "vfd_create_batch")
        self._h = h
        self._maps: list = []
        self._counts = [0] * len(descs)
        self.scene_count = len(descs)

    # lifetime
    def close(self):
        if getattr(self, "_h", None):
            lib().vfd_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # setters
    def SetDescription(self, desc: vfd_desc | dict):
        d = desc if isinstance(desc, vfd_desc) else make_desc(**desc)
        _check(lib().vfd_set_description(self._h, C.byref(d)), "vfd_set_description")

    def SetFluidObjects(self, positions, velocities=None, scene: int = 0):
        """Concatenated positions (n, 3) and velocities (n, 3) of all fluid objects."""
        x, xp = _f32(np.asarray(positions).reshape(-1, 3))
        vp = None
        if velocities is not None:
            v, vp = _f32(np.asarray(velocities).reshape(-1, 3))
        _check(lib().vfd_scene_set_fluid(self._h, scene, xp, vp, len(x)), "vfd_scene_set_fluid")
        self._counts[scene] = len(x)

    def SetRigidBodies(self, maps: list, scene: int = 0):
        """One VolumeMap per rigid body, in order (replaces the scene's bodies when scene == 0 of a plain sim)."""
        if self.scene_count == 1:
            _check(lib().vfd_clear_rigid_bodies(self._h), "vfd_clear_rigid_bodies")
        for m in maps:
            self.AddRigidBody(m, scene)

    def AddRigidBody(self, vmap: VolumeMap, scene: int = 0):
        self._maps.append(vmap)
        _check(lib().vfd_scene_add_rigid_body(self._h, scene, C.byref(vmap.struct)), "vfd_scene_add_rigid_body")

    def SetPositionMode(self, cell_relative: bool):
        """Absolute FP32 positions (the reference's) or cell-relative ones; restarts the run."""
        _check(lib().vfd_set_position_mode(self._h, _abi.VFD_POSITIONS_CELL_RELATIVE if cell_relative
                                           else _abi.VFD_POSITIONS_ABSOLUTE), "vfd_set_position_mode")

    def Emit(self, positions, velocities=None):
        """Appends particles to the running state (vfd_emit)."""
        x, xp = _f32(positions)
        v, vp = _f32(velocities) if velocities is not None else (None, None)
        _check(lib().vfd_emit(self._h, xp, vp, len(x)), "vfd_emit")

    def SetKernelMode(self, analytic: bool):
        """VFD_KERNEL_ANALYTIC (the spline at |r|, smooth in r) or the reference's tables."""
        mode = _abi.VFD_KERNEL_ANALYTIC if analytic else _abi.VFD_KERNEL_TABLE
        _check(lib().vfd_set_kernel_mode(self._h, mode), "vfd_set_kernel_mode")

    def SetGraphMode(self, enabled: bool):
        _check(lib().vfd_set_graph_mode(self._h, int(bool(enabled))), "vfd_set_graph_mode")

    def GetGraphMode(self) -> tuple[bool, bool]:
        """(graphs requested, steps so far ran from graphs)."""
        req, act = C.c_int32(), C.c_int32()
        _check(lib().vfd_get_graph_mode(self._h, C.byref(req), C.byref(act)), "vfd_get_graph_mode")
        return bool(req.value), bool(act.value)

    # stepping
    def Reset(self):
        _check(lib().vfd_reset(self._h), "vfd_reset")

    def OnUpdate(self) -> dict:
        st = vfd_step_stats()
        _check(lib().vfd_step(self._h, C.byref(st)), "vfd_step")
        return st.as_dict()

    def Steps(self, count: int) -> dict:
        st = vfd_step_stats()
        _check(lib().vfd_steps(self._h, count, C.byref(st)), "vfd_steps")
        return st.as_dict()

    def StepsAsync(self, count: int):
        _check(lib().vfd_steps_async(self._h, count), "vfd_steps_async")

    def Synchronize(self) -> dict:
        st = vfd_step_stats()
        _check(lib().vfd_synchronize(self._h, C.byref(st)), "vfd_synchronize")
        return st.as_dict()

    def Simulate(self, on_frame=None) -> int:
        """Runs FrameCount frames from the initial state; on_frame(index, x, v, a, max_v2, dt)."""
        frames = [0]

        def cb(idx, n, x, v, a, mv, dt, user):
            frames[0] += 1
            if on_frame is not None:
                on_frame(idx, np.ctypeslib.as_array(x, (n, 3)).copy(), np.ctypeslib.as_array(v, (n, 3)).copy(),
                         np.ctypeslib.as_array(a, (n, 3)).copy(), mv, dt)

        fn = FRAME_CALLBACK(cb)
        _check(lib().vfd_simulate(self._h, fn, None), "vfd_simulate")
        return frames[0]

    # getters
    def GetParticleCount(self) -> int:
        n = C.c_uint32()
        _check(lib().vfd_get_particle_count(self._h, C.byref(n)), "vfd_get_particle_count")
        return n.value

    def GetParticleRadius(self) -> float:
        return self.GetInfo()["ParticleRadius"]

    def GetCurrentTimeStepSize(self) -> float:
        dt = C.c_float()
        _check(lib().vfd_get_current_time_step_size(self._h, C.byref(dt)), "vfd_get_current_time_step_size")
        return dt.value

    def GetMaxVelocityMagnitude(self) -> float:
        v = C.c_float()
        _check(lib().vfd_get_max_velocity_magnitude(self._h, C.byref(v)), "vfd_get_max_velocity_magnitude")
        return v.value

    def GetDescription(self) -> dict:
        d = vfd_desc()
        _check(lib().vfd_get_description(self._h, C.byref(d)), "vfd_get_description")
        return _abi.desc_to_dict(d)

    def GetInfo(self) -> dict:
        i = vfd_info()
        _check(lib().vfd_get_info(self._h, C.byref(i)), "vfd_get_info")
        return i.as_dict()

    def GetDebugInfo(self, scene: int = 0) -> dict:
        st = vfd_step_stats()
        _check(lib().vfd_scene_get_stats(self._h, scene, C.byref(st)), "vfd_scene_get_stats")
        return st.as_dict()

    def GetKernel(self):
        w = np.zeros(10000, np.float32)
        g = np.zeros(10001, np.float32)
        r, wz = C.c_float(), C.c_float()
        _check(lib().vfd_get_kernel_table(self._h, _fptr(w), _fptr(g), C.byref(r), C.byref(wz)),
               "vfd_get_kernel_table")
        return dict(W=w, GradW=g, radius=r.value, w_zero=wz.value)

    def _n(self, scene: int = 0) -> int:
        # a single scene can grow (Emit) and shrink back (Reset, Simulate): ask the library
        if len(self._counts) == 1:
            return self.GetParticleCount()
        return self._counts[scene]

    def GetState(self, scene: int = 0):
        n = self._n(scene)
        x = np.zeros((n, 3), np.float32)
        v = np.zeros((n, 3), np.float32)
        a = np.zeros((n, 3), np.float32)
        _check(lib().vfd_scene_get_state(self._h, scene, _fptr(x), _fptr(v), _fptr(a)), "vfd_scene_get_state")
        return x, v, a

    def GetStateInto(self, x=None, v=None, a=None, scene: int = 0):
        """GetState into caller arrays (float32, C-contiguous, (n, 3)), e.g. pinned host memory."""
        n = self._n(scene)
        for arr in (x, v, a):
            if arr is not None and (arr.dtype != np.float32 or not arr.flags.c_contiguous or arr.size != 3 * n):
                raise ValueError(f"arrays must be C-contiguous float32 of shape ({n}, 3)")
        _check(lib().vfd_scene_get_state(self._h, scene, _fptr(x), _fptr(v), _fptr(a)), "vfd_scene_get_state")

    def SetState(self, x=None, v=None):
        xp = vp = None
        n = self._n(0)
        if x is not None:
            xa, xp = _f32(np.asarray(x).reshape(-1, 3))
            if len(xa) != n:
                raise ValueError(f"SetState: {len(xa)} positions for {n} particles")
        if v is not None:
            va, vp = _f32(np.asarray(v).reshape(-1, 3))
            if len(va) != n:
                raise ValueError(f"SetState: {len(va)} velocities for {n} particles")
        _check(lib().vfd_set_state(self._h, xp, vp), "vfd_set_state")

    def Checkpoint(self) -> bytes:
        """The carried state (positions, velocities, viscosity warm start, temporal
        curvature, accelerations, original indices) and the solver clock (dt, frame
        time, iteration) as an opaque image for Restore."""
        size = C.c_uint64(0)
        _check(lib().vfd_checkpoint_size(self._h, C.byref(size)), "vfd_checkpoint_size")
        buf = C.create_string_buffer(size.value)
        _check(lib().vfd_checkpoint(self._h, buf, size.value), "vfd_checkpoint")
        return buf.raw

    def Restore(self, image: bytes):
        """Continues from a Checkpoint image of a simulation with the same scenes,
        particle counts and modes; the next steps repeat the checkpointed run's."""
        buf = C.create_string_buffer(bytes(image), len(image))
        _check(lib().vfd_restore(self._h, buf, len(image)), "vfd_restore")

    def GetField(self, field: int, body: int = 0) -> np.ndarray:
        n = self._n(0)
        shape = (n, 3) if field in _abi.VECTOR_FIELDS else (n,)
        out = np.zeros(shape, np.float32)
        _check(lib().vfd_get_field(self._h, field, body, _fptr(out)), "vfd_get_field")
        return out

    # adjoint (no counterpart in the reference)
    def AdjointForward(self, steps: int, checkpoint_every: int = 10) -> dict:
        """`steps` steps from the current state, checkpointed for AdjointBackward."""
        st = vfd_step_stats()
        _check(lib().vfd_adjoint_forward(self._h, steps, checkpoint_every, C.byref(st)), "vfd_adjoint_forward")
        return st.as_dict()

    def AdjointBackward(self, x_bar, v_bar):
        """Cotangents of the final (x, v) -> those of the initial (x, v) and of
        (Viscosity, BoundaryViscosity), for the run of the last AdjointForward."""
        n = self.GetParticleCount()
        xb, xbp = _f32(np.asarray(x_bar).reshape(n, 3))
        vb, vbp = _f32(np.asarray(v_bar).reshape(n, 3))
        x0 = np.empty((n, 3), np.float32)
        v0 = np.empty((n, 3), np.float32)
        pb = np.zeros(2, np.float32)
        _check(lib().vfd_adjoint_backward(self._h, xbp, vbp, x0.ctypes.data_as(C.POINTER(C.c_float)),
                                          v0.ctypes.data_as(C.POINTER(C.c_float)),
                                          pb.ctypes.data_as(C.POINTER(C.c_float))), "vfd_adjoint_backward")
        return x0, v0, pb

    def AdjointRelease(self):
        _check(lib().vfd_adjoint_release(self._h), "vfd_adjoint_release")

    def AdjointSetWarmStart(self, mode: int):
        """Initial guess of the adjoint viscosity solves: _abi.WARM_COLD, WARM_PREVIOUS (the
        default) or WARM_EXTRAPOLATE."""
        _check(lib().vfd_adjoint_set_warm_start(self._h, int(mode)), "vfd_adjoint_set_warm_start")

    def AdjointSetTolerance(self, factor: float):
        """Tolerance of the adjoint viscosity solves relative to the forward's (0, 1]; default 1."""
        _check(lib().vfd_adjoint_set_tolerance(self._h, float(factor)), "vfd_adjoint_set_tolerance")

    def AdjointStats(self) -> dict:
        """Counters of the last AdjointBackward (steps, replayed steps, viscosity solves and
        their CG iterations)."""
        st = _abi.vfd_adjoint_stats()
        _check(lib().vfd_adjoint_get_stats(self._h, C.byref(st)), "vfd_adjoint_get_stats")
        return st.as_dict()

    def ProfileKernels(self, steps: int) -> dict:
        """{kernel name: (launches, total ms)} over `steps` eagerly launched steps."""
        cap = 64
        arr = (vfd_kernel_time * cap)()
        cnt = C.c_uint32()
        _check(lib().vfd_profile_kernels(self._h, steps, arr, cap, C.byref(cnt)), "vfd_profile_kernels")
        return {arr[i].name.decode(): (arr[i].launches, arr[i].total_ms) for i in range(cnt.value)}

    def Autotune(self, steps: int = 2) -> dict:
        """Per-kernel lanes per particle chosen by timing (state restored afterwards)."""
        arr = (C.c_uint8 * 16)()
        _check(lib().vfd_autotune(self._h, steps, arr, 16), "vfd_autotune")
        return {k: arr[i] for i, k in enumerate(TUNED_KERNELS)}

    def SetLanes(self, lanes):
        arr = (C.c_uint8 * len(lanes))(*lanes)
        _check(lib().vfd_set_lanes(self._h, arr, len(lanes)), "vfd_set_lanes")

    def GetLanes(self) -> list:
        arr = (C.c_uint8 * 16)()
        _check(lib().vfd_get_lanes(self._h, arr, 16), "vfd_get_lanes")
        return list(arr)[:len(TUNED_KERNELS)]

    def SetPrecision(self, fp64: bool):
        """FP64 (the whole step in double on the GPU, a reference trajectory) or the
        default FP32 step; restarts from the fluid objects."""
        _check(lib().vfd_set_precision(self._h, 1 if fp64 else 0), "vfd_set_precision")

    def GetStateF64(self):
        """Positions and velocities of the FP64 path as float64 arrays (n, 3)."""
        n = self._n(0)
        x = np.zeros((n, 3), np.float64)
        v = np.zeros((n, 3), np.float64)
        dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
        _check(lib().vfd_get_state_f64(self._h, dp(x), dp(v)), "vfd_get_state_f64")
        return x, v

    def SetTiles(self, tiles):
        """Per solver-loop pass, in TUNED_KERNELS order: 0 = walk neighbour rows (gradW / r
        from the density pass's stream), 1 = walk neighbour rows forming gradW / r from the
        table, 3 or 4 = log2 of the cells per shared-memory tile (2x2x2, 4x2x2); entries of
        other kernels are ignored."""
        arr = (C.c_uint8 * len(tiles))(*tiles)
        _check(lib().vfd_set_tiles(self._h, arr, len(tiles)), "vfd_set_tiles")

    def GetTiles(self) -> dict:
        """Tile choice of the three solver-loop passes (0 = neighbour rows, 3 or 4 = log2
        of the cells per tile)."""
        arr = (C.c_uint8 * 16)()
        _check(lib().vfd_get_tiles(self._h, arr, 16), "vfd_get_tiles")
        return {k: arr[i] for i, k in enumerate(TUNED_KERNELS) if k in TILE_KERNELS}

    def SetBlocks(self, blocks):
        """Threads per block (64, 128, 256) of the neighbour-row kernels, TUNED_KERNELS order."""
        arr = (C.c_uint16 * len(blocks))(*blocks)
        _check(lib().vfd_set_blocks(self._h, arr, len(blocks)), "vfd_set_blocks")

    def GetBlocks(self) -> dict:
        arr = (C.c_uint16 * 16)()
        _check(lib().vfd_get_blocks(self._h, arr, 16), "vfd_get_blocks")
        return {k: arr[i] for i, k in enumerate(TUNED_KERNELS)}

    def GetStream(self) -> int:
        p = C.c_void_p()
        _check(lib().vfd_get_stream(self._h, C.byref(p)), "vfd_get_stream")
        return p.value or 0

    def GetLaunchCount(self, reset: bool = False) -> int:
        c = C.c_uint64()
        _check(lib().vfd_get_launch_count(self._h, C.byref(c), int(reset)), "vfd_get_launch_count")
        return c.value

    def FindNeighbors(self):
        _check(lib().vfd_find_neighbors(self._h), "vfd_find_neighbors")

    def GetNeighbors(self) -> dict:
        n = self._n(0)
        counts = np.zeros(n, np.uint32)
        offsets = np.zeros(n, np.uint32)
        sort_idx = np.zeros(n, np.uint32)
        keys = np.zeros(n, np.uint32)
        total = C.c_uint32()
        _check(lib().vfd_get_neighbors(self._h, _u32ptr(counts), _u32ptr(offsets), None, 0, C.byref(total),
                                       _u32ptr(sort_idx), _u32ptr(keys)), "vfd_get_neighbors")
        lst = np.zeros(max(1, total.value), np.uint32)
        _check(lib().vfd_get_neighbors(self._h, None, None, _u32ptr(lst), total.value, C.byref(total), None, None),
               "vfd_get_neighbors")
        return dict(counts=counts, offsets=offsets, list=lst[:total.value], sort_indices=sort_idx, cell_keys=keys)


def find_neighbors_noalloc(xyz_ptr: int, n: int, particle_radius: float, counts_ptr: int, neighbors_ptr: int,
                           sort_indices_ptr: int, stream: int = 0) -> int:
    """vfd_find_neighbors_noalloc on caller-owned device buffers (raw device pointers).

    For callers that cannot allocate device memory; the library uses a fixed
    internal device array instead (at most 16384 particles per call). Returns the
    status code (VFD_OK = 0)."""
    return lib().vfd_find_neighbors_noalloc(xyz_ptr, n, C.c_float(particle_radius), counts_ptr, neighbors_ptr,
                                            sort_indices_ptr, stream or None)


def batch_simulation(scene_list: list, maps: list | None = None) -> DFSPHSimulation:
    """One DFSPHSimulation advancing every vfd_gb300.scenes scene of `scene_list` together
    (volume maps built on the GPU unless given as one list of maps per scene)."""
    sim = DFSPHSimulation(scenes=[make_desc(**s["desc"]) for s in scene_list])
    for k, s in enumerate(scene_list):
        sim.SetFluidObjects(s["x"], s["v"], scene=k)
        r = s["desc"]["ParticleRadius"]
        ms = maps[k] if maps is not None else [
            build_box_map(b["min"], b["max"], b["inverted"], b["padding"], b["resolution"], r) for b in s["boxes"]]
        for m in ms:
            sim.AddRigidBody(m, scene=k)
    return sim


def scene_simulation(scene: dict, desc_overrides: dict | None = None, maps: list | None = None) -> DFSPHSimulation:
    """A DFSPHSimulation loaded with a vfd_gb300.scenes scene (volume maps built on the GPU unless given)."""
    d = dict(scene["desc"])
    if desc_overrides:
        d.update(desc_overrides)
    sim = DFSPHSimulation(make_desc(**d))
    sim.SetFluidObjects(scene["x"], scene["v"])
    if maps is None:
        r = d["ParticleRadius"]
        maps = [build_box_map(b["min"], b["max"], b["inverted"], b["padding"], b["resolution"], r)
                for b in scene["boxes"]]
    for m in maps:
        sim.AddRigidBody(m)
    return sim
