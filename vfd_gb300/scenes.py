"""Seeded synthetic scenes for the DFSPH step.

The reference samples fluid volumes from meshes in its editor
(FluidObject/FluidObject.cpp:6-25, Utility/Sampler/ParticleSampler.cpp:7-91)
and builds rigid bodies from meshes (RigidBody/RigidBody.cu:10-72). No
dataset is involved; these generators produce lattice blocks, spheres and
boxes of the sizes the benchmark configurations name, from a SplitMix64
stream so that every run of a configuration sees the same particles.

Every scene is a dict:
  x      float32 (n, 3) positions
  v      float32 (n, 3) velocities
  desc   dict of vfd_desc overrides (reference field names)
  boxes  list of dicts(min, max, inverted, padding, resolution): rigid bodies,
         each turned into a volume map (vfd_build_box_map)
  name   short label
"""
from __future__ import annotations

import math

import numpy as np

_MASK = (1 << 64) - 1


class SplitMix64:
    """SplitMix64 (Steele, Lea, Flood 2014), the seed stream of every scene."""

    def __init__(self, seed: int):
        self.state = seed & _MASK

    def next_u64(self) -> int:
        self.state = (self.state + 0x9E3779B97F4A7C15) & _MASK
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _MASK
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _MASK
        return z ^ (z >> 31)

    def uniform(self, n: int) -> np.ndarray:
        """n doubles in [0, 1) from the top 53 bits, vectorised over a block of draws."""
        out = np.empty(n, dtype=np.float64)
        # vectorised SplitMix64: states s_k = s_0 + k * gamma
        gamma = np.uint64(0x9E3779B97F4A7C15)
        k = np.arange(1, n + 1, dtype=np.uint64)
        with np.errstate(over="ignore"):
            z = np.uint64(self.state) + k * gamma
            z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
            z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
            z = z ^ (z >> np.uint64(31))
        self.state = (self.state + n * 0x9E3779B97F4A7C15) & _MASK
        out[:] = (z >> np.uint64(11)).astype(np.float64) * (1.0 / (1 << 53))
        return out


def config_seed(config: int) -> int:
    return 0x5EED0000 + config


def lattice_block(counts, r, origin, jitter_frac, rng: SplitMix64) -> np.ndarray:
    """counts = (nx, ny, nz) particles at spacing 2r; first centre at origin + r;
    each component jittered by U(-jitter_frac*r, +jitter_frac*r)."""
    nx, ny, nz = (int(c) for c in counts)
    ix, iy, iz = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    idx = np.stack([ix.ravel(), iy.ravel(), iz.ravel()], axis=1).astype(np.float64)
    # order: x slowest ... z fastest, like a nested x/y/z loop
    pos = np.asarray(origin, dtype=np.float64) + r + idx * (2.0 * r)
    if jitter_frac > 0:
        u = rng.uniform(pos.size).reshape(pos.shape)
        pos = pos + (2.0 * u - 1.0) * (jitter_frac * r)
    return pos.astype(np.float32)


def lattice_sphere(center, radius, r, jitter_frac, rng: SplitMix64) -> np.ndarray:
    """Lattice points (spacing 2r) inside a sphere."""
    n = int(math.ceil(radius / (2.0 * r))) + 1
    g = np.arange(-n, n + 1, dtype=np.float64) * (2.0 * r)
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    pts = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    pts = pts[np.einsum("ij,ij->i", pts, pts) <= radius * radius]
    if jitter_frac > 0:
        u = rng.uniform(pts.size).reshape(pts.shape)
        pts = pts + (2.0 * u - 1.0) * (jitter_frac * r)
    return (pts + np.asarray(center, dtype=np.float64)).astype(np.float32)


# With padding 0 (the reference's scene default), a volume map's collision
# surface lies r inside the mesh surface (distance field sign*(sd - (padding - r)),
# RigidBody.cu:28-42), and a particle is in equilibrium about 2r from that
# surface. Lattices therefore start with their first centre 3r from a wall.
def wall_gap(r: float) -> float:
    """Gap between a wall and the first lattice cell (its centre sits at gap + r)."""
    return 2.0 * r


def container(bmin, bmax, r, resolution=(20, 20, 20)) -> dict:
    """An inverted box (fluid inside), padding 0."""
    return dict(min=tuple(float(v) for v in bmin), max=tuple(float(v) for v in bmax),
                inverted=True, padding=0.0, resolution=tuple(int(v) for v in resolution))


def solid_box(bmin, bmax, r, resolution=(20, 20, 20)) -> dict:
    """A solid box (fluid outside), padding 0."""
    return dict(min=tuple(float(v) for v in bmin), max=tuple(float(v) for v in bmax),
                inverted=False, padding=0.0, resolution=tuple(int(v) for v in resolution))


# Solver settings shared by the benchmark configurations. The reference's
# defaults have MinPressureSolverIterations = MinDivergenceSolverIterations = 0;
# its while loops (DFSPHImplementation.cu:461, :532) start from error 0, so with
# a minimum of 0 they never run. A minimum of 2 (the original DFSPH
# implementation's default) makes the 0.1 % density-error bound effective.
SOLVER = dict(MinPressureSolverIterations=2, MinDivergenceSolverIterations=2,
              MaxPressureSolverError=10.0, MaxDivergenceSolverError=10.0)


def dam_break_8k(n_side: int = 20, box_scale=(1.0, 1.0, 1.0), seed: int | None = None,
                 map_resolution=(20, 20, 20)) -> dict:
    """The 8,000-particle dam break: n_side^3 block (20^3), r = 0.025, jitter +-0.05 r, in the corner
    of a closed box. A 20^3 block at spacing 2r is 1 m wide, so the box edge is
    the block edge plus the wall gaps (1.1 m); box_scale = (2, 1, 1) is the
    dam-break variant c1b. No viscosity, no surface tension."""
    r = 0.025
    rng = SplitMix64(config_seed(1) if seed is None else seed)
    g = wall_gap(r)
    x = lattice_block((n_side, n_side, n_side), r, (g, g, g), 0.05, rng)
    edge = n_side * 2.0 * r + 2.0 * g
    box = tuple(s * edge for s in box_scale)
    desc = dict(ParticleRadius=r, EnableViscositySolver=0, EnableSurfaceTensionSolver=0,
                Viscosity=0.0, BoundaryViscosity=0.0, **SOLVER)
    return dict(name=f"dam_break_{len(x)}", x=x, v=np.zeros_like(x), desc=desc,
                boxes=[container((0, 0, 0), box, r, map_resolution)])


def viscous_dam_break(n_side: int = 100, r: float = 0.005, seed: int | None = None,
                      map_resolution=None) -> dict:
    """The 1M-particle high-viscosity dam break: n_side^3 jittered lattice (100^3 = 1M at r = 0.005, a 1 m block)
    in a box of 2 x 1.5 x 1 block edges; dynamic viscosity 50 Pa s
    (Viscosity = 0.05), boundary viscosity 0.05, CG tolerance 1e-4 relative
    (MaxViscositySolverError = 0.01), surface tension 0.05, CSD 10000."""
    rng = SplitMix64(config_seed(2) if seed is None else seed)
    g = wall_gap(r)
    x = lattice_block((n_side, n_side, n_side), r, (g, g, g), 0.05, rng)
    edge = n_side * 2.0 * r
    box = (2.0 * edge + 2.0 * g, 1.5 * edge + 2.0 * g, 1.0 * edge + 2.0 * g)
    if map_resolution is None:
        map_resolution = (40, 30, 20)
    desc = dict(ParticleRadius=r, Viscosity=0.05, BoundaryViscosity=0.05, MaxViscositySolverError=0.01,
                EnableViscositySolver=1, EnableSurfaceTensionSolver=1, SurfaceTension=0.05, CSD=10000,
                **SOLVER)
    return dict(name=f"viscous_dam_break_{len(x)}", x=x, v=np.zeros_like(x), desc=desc,
                boxes=[container((0, 0, 0), box, r, map_resolution)])


def falling_drop(n_target: int, r: float, viscosity: float, rng: SplitMix64) -> dict:
    radius = 2.0 * r * (3.0 * n_target / (4.0 * math.pi)) ** (1.0 / 3.0)
    box = (4.0 * radius, 6.0 * radius, 4.0 * radius)  # the drop falls 2 radii onto the floor
    x = lattice_sphere((2.0 * radius, 3.0 * radius, 2.0 * radius), radius, r, 0.05, rng)
    desc = dict(ParticleRadius=r, Viscosity=viscosity, BoundaryViscosity=viscosity, MaxViscositySolverError=0.01,
                EnableViscositySolver=1, EnableSurfaceTensionSolver=0, **SOLVER)
    return dict(name=f"drop_{len(x)}", x=x, v=np.zeros_like(x), desc=desc,
                boxes=[container((0, 0, 0), box, r, (16, 16, 16))])


def block_dam_break(n_target: int, r: float, viscosity: float, rng: SplitMix64) -> dict:
    nx = max(4, int(round(n_target ** (1.0 / 3.0))))
    ny = max(4, int(round(n_target / (nx * nx))))
    g = wall_gap(r)
    x = lattice_block((nx, ny, nx), r, (g, g, g), 0.05, rng)
    ex, ey = nx * 2.0 * r + g, ny * 2.0 * r + g
    box = (2.0 * ex, 1.5 * ey, 2.0 * ex)  # the block covers a quarter of the footprint
    desc = dict(ParticleRadius=r, Viscosity=viscosity, BoundaryViscosity=viscosity, MaxViscositySolverError=0.01,
                EnableViscositySolver=1, EnableSurfaceTensionSolver=0, **SOLVER)
    return dict(name=f"block_{len(x)}", x=x, v=np.zeros_like(x), desc=desc,
                boxes=[container((0, 0, 0), box, r, (16, 16, 16))])


def uneven_batch(count: int = 256, r: float = 0.005, n_min: int = 2000, n_max: int = 64000,
                 seed: int | None = None) -> list[dict]:
    """The uneven batch: `count` independent scenes, particle counts log-uniform in
    [n_min, n_max], even = dam break, odd = falling drop, dynamic viscosity
    log-uniform in [0.01, 100] Pa s (Viscosity = mu / 1000)."""
    rng = SplitMix64(config_seed(3) if seed is None else seed)
    u = rng.uniform(2 * count)
    scenes = []
    for i in range(count):
        n = int(math.floor(math.exp(math.log(n_min) + u[2 * i] * (math.log(n_max) - math.log(n_min)))))
        mu = math.exp(math.log(0.01) + u[2 * i + 1] * (math.log(100.0) - math.log(0.01)))
        sub = SplitMix64(config_seed(3) * 1000 + i)
        s = block_dam_break(n, r, mu / 1000.0, sub) if i % 2 == 0 else falling_drop(n, r, mu / 1000.0, sub)
        scenes.append(s)
    return scenes


def viscous_drop_33k(r: float = 0.0025, radius: float = 0.1, seed: int | None = None) -> dict:
    """The differentiable viscous drop: sphere of radius 0.1 m at spacing 2r (r = 0.0025 gives ~33k
    particles), 0.3 m above a floor, velocity = 8 seeded Fourier modes scaled to
    max 0.5 m/s, dynamic viscosity 10 Pa s (Viscosity = 0.01)."""
    rng = SplitMix64(config_seed(4) if seed is None else seed)
    center = (0.3, 0.3 + 0.05, 0.3)
    x = lattice_sphere(center, radius, r, 0.05, rng)
    params = rng.uniform(8 * 7)
    v = np.zeros_like(x, dtype=np.float64)
    for m in range(8):
        p = params[7 * m: 7 * m + 7]
        kmag = 2 * math.pi / 0.2 + p[0] * (2 * math.pi / 0.05 - 2 * math.pi / 0.2)
        th, ph = math.acos(2 * p[1] - 1), 2 * math.pi * p[2]
        k = kmag * np.array([math.sin(th) * math.cos(ph), math.sin(th) * math.sin(ph), math.cos(th)])
        amp = np.array([p[3], p[4], p[5]]) * 2 - 1
        phase = 2 * math.pi * p[6]
        v += np.sin(x.astype(np.float64) @ k + phase)[:, None] * amp[None, :]
    v *= 0.5 / max(1e-12, np.linalg.norm(v, axis=1).max())
    desc = dict(ParticleRadius=r, Viscosity=0.01, BoundaryViscosity=0.01, MaxViscositySolverError=0.01,
                EnableViscositySolver=1, EnableSurfaceTensionSolver=0, **SOLVER)
    floor = solid_box((0.0, 0.0, 0.0), (0.6, 0.05, 0.6), r, (20, 8, 20))
    return dict(name=f"viscous_drop_{len(x)}", x=x, v=v.astype(np.float32), desc=desc, boxes=[floor])


def jet_coiling_8m(pool=(400, 50, 400), r: float = 0.0015, seed: int | None = None,
                   map_resolution=(40, 24, 40)) -> dict:
    """The 8M-particle jet-coiling scene: a viscous jet (inflow disk of radius 0.02 m at 1 m/s, downwards, 0.5 m
    above the floor) onto a resting pool. The inflow alone adds ~140 particles per layer
    (about 5e4 per second of flow), far from 8M, so a pool of pool[0] x pool[1] x pool[2]
    particles (400 x 50 x 400 = 8M at spacing 2r = 3 mm: 1.2 x 0.15 x 1.2 m) rests on
    the floor of a closed box and the jet falls 0.35 m onto it. Kinematic viscosity 0.2
    (200 Pa s), surface tension 0.07, 2000 steps. Returns the scene and the emitter's
    parameters (center, direction, radius, speed)."""
    rng = SplitMix64(config_seed(5) if seed is None else seed)
    g = wall_gap(r)
    x = lattice_block(pool, r, (g, g, g), 0.05, rng)
    edge = [c * 2.0 * r + 2.0 * g for c in pool]
    box = (edge[0], 0.8, edge[2])
    desc = dict(ParticleRadius=r, Viscosity=0.2, BoundaryViscosity=0.2, MaxViscositySolverError=0.01,
                EnableViscositySolver=1, EnableSurfaceTensionSolver=1, SurfaceTension=0.07, **SOLVER)
    inflow = dict(center=(0.5 * box[0], 0.5, 0.5 * box[2]), direction=(0.0, -1.0, 0.0), radius=0.02, speed=1.0)
    return dict(name=f"jet_coiling_{len(x)}", x=x, v=np.zeros_like(x), desc=desc,
                boxes=[container((0.0, 0.0, 0.0), box, r, map_resolution)], inflow=inflow)


def small_dam_break(n_side: int = 12, r: float = 0.025, viscosity: float = 0.0, surface_tension: float = 0.0,
                    seed: int = 7, box_scale=(2.0, 1.5, 1.0), map_resolution=(24, 18, 12)) -> dict:
    """A small dam break for parity tests (all features switchable)."""
    rng = SplitMix64(seed)
    g = wall_gap(r)
    x = lattice_block((n_side, n_side, n_side), r, (g, g, g), 0.05, rng)
    edge = n_side * 2.0 * r + 2.0 * g
    box = tuple(s * edge for s in box_scale)
    desc = dict(ParticleRadius=r, Viscosity=viscosity, BoundaryViscosity=viscosity,
                EnableViscositySolver=int(viscosity > 0), EnableSurfaceTensionSolver=int(surface_tension > 0),
                SurfaceTension=surface_tension, MaxViscositySolverError=0.01, **SOLVER)
    return dict(name=f"small_dam_break_{len(x)}", x=x, v=np.zeros_like(x), desc=desc,
                boxes=[container((0, 0, 0), box, r, map_resolution)])


def jet_column_8m(pool=(400, 50, 400), r: float = 0.0015, offset=(0.0, 0.0, 0.0), seed: int | None = None) -> dict:
    """The jet-coiling scene with its jet already flowing: the resting pool of
    jet_coiling_8m plus the column the inflow would have emitted, disk layers of spacing
    2r from the inflow disk (0.5 m) down to 4r above the pool, moving at the inflow
    velocity (1 m/s down). It needs no emitter, so every arithmetic mode (FP32 absolute,
    FP32 cell-relative, FP64) starts from the same particles and keeps them. `offset`
    translates the whole scene (boxes included)."""
    from .emitter import InflowEmitter
    s = jet_coiling_8m(pool=pool, r=r, seed=seed)
    f = s["inflow"]
    em = InflowEmitter(f["center"], f["direction"], f["radius"], f["speed"], r)
    top = float(s["x"][:, 1].max()) + 4.0 * r
    layers = int((f["center"][1] - top) / (2.0 * r))
    xs, vs = zip(*(em.layer(k * 2.0 * r) for k in range(layers)))
    off = np.asarray(offset, np.float64)
    x = (np.concatenate([s["x"], *xs]).astype(np.float64) + off).astype(np.float32)
    v = np.concatenate([s["v"], *vs]).astype(np.float32)
    boxes = [dict(b, min=tuple(np.asarray(b["min"]) + off), max=tuple(np.asarray(b["max"]) + off)) for b in s["boxes"]]
    return dict(s, name=f"jet_column_{len(x)}", x=x, v=v, boxes=boxes)
