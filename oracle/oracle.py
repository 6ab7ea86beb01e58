"""ctypes wrapper of the CPU oracle (oracle/dfsph_oracle.cpp).

TEST INFRASTRUCTURE ONLY: tests, __graft_entry__.smoke() and bench.py's CPU
baseline use it as the checker and the timed CPU restatement of the
reference's DFSPH step. The product (vfd_gb300) never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

from vfd_gb300 import _abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libvfd_oracle.so")

_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (seconds)."""
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < max(
            os.path.getmtime(os.path.join(HERE, "dfsph_oracle.cpp")),
            os.path.getmtime(os.path.join(HERE, "sph_oracle.cpp")),
            os.path.getmtime(os.path.join(HERE, "..", "include", "vfd_dfsph.h")),
            os.path.getmtime(os.path.join(HERE, "..", "include", "vfd_sph.h"))):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = C.CDLL(LIB_PATH)
            P = C.c_void_p
            u32p = C.POINTER(C.c_uint32)
            f32p = C.POINTER(C.c_float)
            f64p = C.POINTER(C.c_double)
            L.orc_create.restype = P
            L.orc_create.argtypes = [C.POINTER(_abi.vfd_desc), C.c_int]
            L.orc_destroy.argtypes = [P]
            L.orc_set_fluid.argtypes = [P, f32p, f32p, C.c_uint32]
            L.orc_add_rigid_body.argtypes = [P, C.POINTER(_abi.vfd_volume_map)]
            L.orc_reset.argtypes = [P]
            L.orc_set_kernel_mode.argtypes = [P, C.c_int]
            L.orc_emit.argtypes = [P, f32p, f32p, C.c_uint32]
            L.orc_step.argtypes = [P, C.POINTER(_abi.vfd_step_stats)]
            L.orc_set_carried.argtypes = [P, f32p, f32p, f32p, f32p, C.c_double]
            L.orc_find_neighbors.argtypes = [P]
            L.orc_get_neighbors.argtypes = [P, u32p, u32p, u32p, C.c_uint32, u32p, u32p, u32p]
            L.orc_get_state.argtypes = [P, f64p, f64p, f64p]
            L.orc_get_field.argtypes = [P, C.c_int, C.c_uint32, f64p]
            L.orc_get_time_step.argtypes = [P, f64p]
            L.orc_kernel_table.argtypes = [C.c_float, f32p, f32p, f32p]
            L.orc_halton.argtypes = [f32p]
            L.orc_morton3.restype = C.c_uint32
            L.orc_morton3.argtypes = [C.c_uint32, C.c_uint32, C.c_uint32]
            L.orc_box_map_sizes.argtypes = [u32p, u32p, u32p]
            L.orc_build_box_map.argtypes = [f32p, f32p, C.c_int, C.c_float, u32p, C.c_float, f32p, u32p, u32p,
                                            C.POINTER(_abi.vfd_volume_map)]
            L.orc_map_interpolate.argtypes = [C.POINTER(_abi.vfd_volume_map), C.c_uint32, f32p, C.c_uint32, f64p,
                                              f64p]
            L.orc_map_interpolate_d.argtypes = [C.POINTER(_abi.vfd_volume_map), C.c_uint32, f64p, C.c_uint32, f64p,
                                                f64p]
            L.orc_gauss_legendre.argtypes = [C.c_uint, f64p, f64p]
            L.orc_build_mesh_map.argtypes = [f32p, C.c_uint32, u32p, C.c_uint32, f32p, C.c_int, C.c_float, u32p,
                                             C.c_float, f32p, u32p, u32p, C.POINTER(_abi.vfd_volume_map)]
            L.orc_mesh_signed_distance.argtypes = [f32p, C.c_uint32, u32p, C.c_uint32, f32p, f32p, C.c_uint32,
                                                   f32p]
            L.orc_sample_mesh_volume.argtypes = [f32p, C.c_uint32, u32p, C.c_uint32, f32p, C.c_float, u32p, C.c_int,
                                                 C.c_int, f32p, C.c_uint32, u32p]
            L.orc_map_node_positions.argtypes = [C.POINTER(_abi.vfd_volume_map), f32p]
            L.orc_set_threads.argtypes = [C.c_int]
            L.orc_get_threads.restype = C.c_int
            _lib = L
    return _lib


def _f32(a):
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a, a.ctypes.data_as(C.POINTER(C.c_float))


def _ptr(a, ctype):
    return a.ctypes.data_as(C.POINTER(ctype)) if a is not None else None


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


def get_threads() -> int:
    return int(lib().orc_get_threads())


def kernel_table(radius: float):
    w = np.zeros(10000, np.float32)
    g = np.zeros(10001, np.float32)
    wz = C.c_float()
    lib().orc_kernel_table(C.c_float(radius), _ptr(w, C.c_float), _ptr(g, C.c_float), C.byref(wz))
    return w, g, wz.value


def halton() -> np.ndarray:
    out = np.zeros(49152, np.float32)
    lib().orc_halton(_ptr(out, C.c_float))
    return out


def gauss_legendre(n: int):
    x = np.zeros(n, np.float64)
    w = np.zeros(n, np.float64)
    lib().orc_gauss_legendre(n, _ptr(x, C.c_double), _ptr(w, C.c_double))
    return x, w


def map_node_positions(vmap) -> np.ndarray:
    out = np.zeros((vmap.struct.node_count, 3), np.float32)
    lib().orc_map_node_positions(C.byref(vmap.struct), _ptr(out, C.c_float))
    return out


def morton3(x: int, y: int, z: int) -> int:
    return int(lib().orc_morton3(x, y, z))


class VolumeMap:
    """Holds the arrays of a vfd_volume_map alive together with the struct."""

    def __init__(self, nodes, cells, cell_map, struct):
        self.nodes, self.cells, self.cell_map, self.struct = nodes, cells, cell_map, struct

    @staticmethod
    def from_arrays(nodes, cells, cell_map, meta) -> "VolumeMap":
        m = _abi.vfd_volume_map()
        nodes = np.ascontiguousarray(nodes, np.float32)
        cells = np.ascontiguousarray(cells, np.uint32)
        cell_map = np.ascontiguousarray(cell_map, np.uint32)
        m.nodes = _ptr(nodes, C.c_float)
        m.cells = _ptr(cells, C.c_uint32)
        m.cell_map = _ptr(cell_map, C.c_uint32)
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
    res = np.ascontiguousarray(resolution, np.uint32)
    nn, nc = C.c_uint32(), C.c_uint32()
    lib().orc_box_map_sizes(_ptr(res, C.c_uint32), C.byref(nn), C.byref(nc))
    nodes = np.zeros(2 * nn.value, np.float32)
    cells = np.zeros(2 * nc.value * 32, np.uint32)
    cell_map = np.zeros(2 * nc.value, np.uint32)
    m = _abi.vfd_volume_map()
    bmin_a, _ = _f32(bmin)
    bmax_a, _ = _f32(bmax)
    lib().orc_build_box_map(_ptr(bmin_a, C.c_float), _ptr(bmax_a, C.c_float), int(bool(inverted)),
                            C.c_float(padding), _ptr(res, C.c_uint32), C.c_float(particle_radius),
                            _ptr(nodes, C.c_float), _ptr(cells, C.c_uint32), _ptr(cell_map, C.c_uint32),
                            C.byref(m))
    return VolumeMap(nodes, cells, cell_map, m)


def _mesh(vertices, triangles, transform):
    v = np.ascontiguousarray(np.asarray(vertices, np.float32).reshape(-1, 3))
    t = np.ascontiguousarray(np.asarray(triangles, np.uint32).reshape(-1, 3))
    col = None if transform is None else np.ascontiguousarray(np.asarray(transform, np.float32).reshape(4, 4).T.reshape(16))
    return v, t, col, (_ptr(col, C.c_float) if col is not None else None)


def build_mesh_map(vertices, triangles, transform=None, inverted: bool = False, padding: float = 0.0,
                   resolution=(20, 20, 20), particle_radius: float = 0.025) -> VolumeMap:
    """RigidBody::RigidBody (RigidBody.cu:10-72) of a triangle mesh, on the CPU."""
    res = np.ascontiguousarray(resolution, np.uint32)
    nn, nc = C.c_uint32(), C.c_uint32()
    lib().orc_box_map_sizes(_ptr(res, C.c_uint32), C.byref(nn), C.byref(nc))
    v, t, col, colp = _mesh(vertices, triangles, transform)
    nodes = np.zeros(2 * nn.value, np.float32)
    cells = np.zeros(2 * nc.value * 32, np.uint32)
    cell_map = np.zeros(2 * nc.value, np.uint32)
    m = _abi.vfd_volume_map()
    rc = lib().orc_build_mesh_map(_ptr(v, C.c_float), len(v), _ptr(t, C.c_uint32), len(t), colp, int(bool(inverted)),
                                  C.c_float(padding), _ptr(res, C.c_uint32), C.c_float(particle_radius),
                                  _ptr(nodes, C.c_float), _ptr(cells, C.c_uint32), _ptr(cell_map, C.c_uint32),
                                  C.byref(m))
    if rc != 0:
        raise ValueError(f"orc_build_mesh_map: {rc}")
    return VolumeMap(nodes, cells, cell_map, m)


def mesh_signed_distance(vertices, triangles, points, transform=None) -> np.ndarray:
    """MeshDistance::SignedDistance (MeshDistance.cpp:187-228) at points, FP32."""
    v, t, col, colp = _mesh(vertices, triangles, transform)
    pts, pp = _f32(points)
    out = np.zeros(len(pts), np.float32)
    rc = lib().orc_mesh_signed_distance(_ptr(v, C.c_float), len(v), _ptr(t, C.c_uint32), len(t), colp, pp, len(pts),
                                        _ptr(out, C.c_float))
    if rc != 0:
        raise ValueError(f"orc_mesh_signed_distance: {rc}")
    return out


def sample_mesh_volume(vertices, triangles, particle_radius: float, resolution=(20, 20, 20), inverted: bool = False,
                       sample_mode: int = 0, transform=None) -> np.ndarray:
    """ParticleSampler::SampleMeshVolume (ParticleSampler.cpp:7-91), on the CPU."""
    v, t, col, colp = _mesh(vertices, triangles, transform)
    res = np.ascontiguousarray(resolution, np.uint32)
    count = C.c_uint32()
    args = (_ptr(v, C.c_float), len(v), _ptr(t, C.c_uint32), len(t), colp, C.c_float(particle_radius),
            _ptr(res, C.c_uint32), int(bool(inverted)), int(sample_mode))
    rc = lib().orc_sample_mesh_volume(*args, None, 0, C.byref(count))
    if rc != 0:
        raise ValueError(f"orc_sample_mesh_volume: {rc}")
    out = np.zeros((count.value, 3), np.float32)
    if count.value:
        lib().orc_sample_mesh_volume(*args, _ptr(out, C.c_float), count.value, C.byref(count))
    return out


def map_interpolate_d(vmap: VolumeMap, field: int, points):
    """FP64 value and gradient of map field `field` at double-precision points (FLT_MAX outside)."""
    pts = np.ascontiguousarray(points, dtype=np.float64)
    n = len(pts)
    phi = np.zeros(n, np.float64)
    grad = np.zeros((n, 3), np.float64)
    lib().orc_map_interpolate_d(C.byref(vmap.struct), field, _ptr(pts, C.c_double), n, _ptr(phi, C.c_double),
                                _ptr(grad, C.c_double))
    return phi, grad


def map_interpolate(vmap: VolumeMap, field: int, points):
    pts, pp = _f32(points)
    n = len(pts)
    phi = np.zeros(n, np.float64)
    grad = np.zeros((n, 3), np.float64)
    lib().orc_map_interpolate(C.byref(vmap.struct), field, pp, n, _ptr(phi, C.c_double), _ptr(grad, C.c_double))
    return phi, grad


class OracleSim:
    """The oracle simulator: precision 32 (FP32 mirror) or 64 (FP64 oracle)."""

    def __init__(self, desc: _abi.vfd_desc, precision: int = 64):
        self._desc = desc
        self.precision = precision
        self.h = lib().orc_create(C.byref(desc), precision)
        if not self.h:
            raise ValueError("orc_create failed")
        self.n = self.n0 = 0
        self._maps = []

    def close(self):
        if self.h:
            lib().orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_fluid(self, x, v=None):
        xa, xp = _f32(x)
        if v is not None:
            va, vp = _f32(v)
        else:
            vp = None
        self.n = self.n0 = len(xa)
        lib().orc_set_fluid(self.h, xp, vp, self.n)

    def add_rigid_body(self, vmap: VolumeMap):
        self._maps.append(vmap)
        rc = lib().orc_add_rigid_body(self.h, C.byref(vmap.struct))
        if rc != 0:
            raise RuntimeError(f"orc_add_rigid_body -> {rc}")

    def reset(self):
        lib().orc_reset(self.h)
        self.n = self.n0

    def emit(self, x, v=None):
        """Appends particles to the running state (as vfd_emit)."""
        xa, xp = _f32(x)
        va, vp = _f32(v) if v is not None else (None, None)
        lib().orc_emit(self.h, xp, vp, len(xa))
        self.n += len(xa)

    def set_kernel_mode(self, analytic: bool):
        """The spline at |r| (analytic) or the reference's tables."""
        lib().orc_set_kernel_mode(self.h, int(bool(analytic)))

    def set_carried(self, x, v, dv=None, dk=None, dt: float = 0.0):
        """Makes the next step start from another run's carried state: positions,
        velocities, viscosity warm start dv, temporal curvature dk and time step dt."""
        xa, xp = _f32(x)
        va, vp = _f32(v)
        dva, dvp = _f32(dv) if dv is not None else (None, None)
        dka, dkp = _f32(np.asarray(dk).reshape(-1)) if dk is not None else (None, None)
        rc = lib().orc_set_carried(self.h, xp, vp, dvp, dkp, float(dt))
        if rc != 0:
            raise ValueError(f"orc_set_carried -> {rc}")

    def step(self) -> dict:
        st = _abi.vfd_step_stats()
        lib().orc_step(self.h, C.byref(st))
        return st.as_dict()

    def find_neighbors(self):
        lib().orc_find_neighbors(self.h)

    def neighbors(self) -> dict:
        n = self.n
        counts = np.zeros(n, np.uint32)
        offsets = np.zeros(n, np.uint32)
        sort_idx = np.zeros(n, np.uint32)
        keys = np.zeros(n, np.uint32)
        total = C.c_uint32()
        lib().orc_get_neighbors(self.h, _ptr(counts, C.c_uint32), _ptr(offsets, C.c_uint32), None, 0,
                                C.byref(total), _ptr(sort_idx, C.c_uint32), _ptr(keys, C.c_uint32))
        lst = np.zeros(max(1, total.value), np.uint32)
        lib().orc_get_neighbors(self.h, None, None, _ptr(lst, C.c_uint32), total.value, C.byref(total), None, None)
        return dict(counts=counts, offsets=offsets, list=lst[:total.value], sort_indices=sort_idx, cell_keys=keys)

    def state(self):
        n = self.n
        x = np.zeros((n, 3), np.float64)
        v = np.zeros((n, 3), np.float64)
        a = np.zeros((n, 3), np.float64)
        lib().orc_get_state(self.h, _ptr(x, C.c_double), _ptr(v, C.c_double), _ptr(a, C.c_double))
        return x, v, a

    def field(self, field: int, body: int = 0) -> np.ndarray:
        n = self.n
        shape = (n, 3) if field in _abi.VECTOR_FIELDS else (n,)
        out = np.zeros(shape, np.float64)
        rc = lib().orc_get_field(self.h, field, body, _ptr(out, C.c_double))
        if rc != 0:
            raise ValueError(f"orc_get_field({field}) -> {rc}")
        return out

    def time_step(self) -> float:
        d = C.c_double()
        lib().orc_get_time_step(self.h, C.byref(d))
        return d.value


def scene_oracle(scene: dict, precision: int = 64, desc_overrides: dict | None = None,
                 maps: list | None = None) -> OracleSim:
    """An OracleSim loaded with a vfd_gb300.scenes scene (maps built on the CPU unless given)."""
    d = dict(scene["desc"])
    if desc_overrides:
        d.update(desc_overrides)
    sim = OracleSim(_abi.make_desc(**d), precision)
    sim.set_fluid(scene["x"], scene["v"])
    if maps is None:
        r = d["ParticleRadius"]
        maps = [build_box_map(b["min"], b["max"], b["inverted"], b["padding"], b["resolution"], r)
                for b in scene["boxes"]]
    for m in maps:
        sim.add_rigid_body(m)
    return sim


class SphOracle:
    """CPU oracle of the legacy SPH pipeline (sph_oracle.cpp), FP32 in the reference's order."""

    def __init__(self, desc, positions):
        L = lib()
        if not getattr(L, "_sph_bound", False):
            from vfd_gb300.sph import vfd_sph_desc, vfd_sph_params
            f32p, u32p = C.POINTER(C.c_float), C.POINTER(C.c_uint32)
            L.orc_sph_create.restype = C.c_void_p
            L.orc_sph_create.argtypes = [C.POINTER(vfd_sph_desc), f32p, C.c_uint32]
            L.orc_sph_destroy.argtypes = [C.c_void_p]
            L.orc_sph_steps.argtypes = [C.c_void_p, C.c_uint32]
            L.orc_sph_set_velocities.argtypes = [C.c_void_p, f32p]
            L.orc_sph_get_state.argtypes = [C.c_void_p, f32p, f32p, f32p, f32p]
            L.orc_sph_get_sort.argtypes = [C.c_void_p, u32p, u32p]
            L.orc_sph_params.argtypes = [C.c_void_p, C.POINTER(vfd_sph_params)]
            L._sph_bound = True
        self.desc = desc
        x, xp = _f32(np.asarray(positions).reshape(-1, 3))
        self.n = len(x)
        self.h = L.orc_sph_create(C.byref(desc), xp, self.n)
        if not self.h:
            raise ValueError("orc_sph_create: invalid description")

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_sph_destroy(self.h)
            self.h = None

    def steps(self, count: int):
        lib().orc_sph_steps(self.h, int(count))

    def set_velocities(self, v):
        va, vp = _f32(np.asarray(v).reshape(-1, 3))
        lib().orc_sph_set_velocities(self.h, vp)

    def state(self):
        x = np.zeros((self.n, 3), np.float32)
        v = np.zeros((self.n, 3), np.float32)
        rho = np.zeros(self.n, np.float32)
        p = np.zeros(self.n, np.float32)
        lib().orc_sph_get_state(self.h, _ptr(x, C.c_float), _ptr(v, C.c_float), _ptr(rho, C.c_float),
                                _ptr(p, C.c_float))
        return x, v, rho, p

    def sort(self):
        k = np.zeros(self.n, np.uint32)
        i = np.zeros(self.n, np.uint32)
        lib().orc_sph_get_sort(self.h, _ptr(k, C.c_uint32), _ptr(i, C.c_uint32))
        return k, i

    def params(self) -> dict:
        from vfd_gb300.sph import vfd_sph_params
        p = vfd_sph_params()
        lib().orc_sph_params(self.h, C.byref(p))
        return {k: (list(getattr(p, k)) if k == "GridSize" else getattr(p, k)) for k, _ in vfd_sph_params._fields_}
