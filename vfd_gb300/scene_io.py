"""Scene files and headless frame output.

`load_scene` reads a scene saved by the reference's Scene::Save (Scene/Scene.cpp:8-45):
a cereal JSON archive ("value0", "value1", ... in order) of an entt registry snapshot,
then "sceneData". The snapshot holds the entity list, then for each component type in
the order Scene::Save names them (ID, Tag, Relationship, Transform, SPHSimulation,
Material, Mesh, RigidBody, FluidObject, DFSPHSimulation) a count followed by that many
(entity, component) pairs. The entity list runs up to the IDComponent count, which is
the value just before the first (entity, component) pair.

`bake` does what the editor's "Bake Objects" button does (Editor/Panels/
ComponentPanel.cpp:608-657) on the GPU: every entity with a FluidObject and a Mesh
component is sampled into particles (vfd_sample_mesh_volume) with its object's
velocity, and every entity with a RigidBody and a Mesh component becomes a volume map
(vfd_build_mesh_map), each placed by its world transform (Scene::
GetWorldSpaceTransformMatrix, Scene/Scene.cpp:277-287: the parent chain of the
Relationship component multiplied from the root). Entities are visited in file order.
The transform is the stored 4x4 matrix (the reference re-composes it from translation,
Euler rotation and scale after loading, which moves it by FP32 rounding).

`save_scene` writes the same layout, so that scenes can be authored here and opened by
the reference. `FrameWriter` is the headless replacement of the frame cache
(DFSPHImplementation.cu:148-167 copies {x, v, a} of every frame to the host for replay):
one .npz file per frame plus an index.
"""
from __future__ import annotations

import json
import os

import numpy as np

from . import _abi
from .meshes import load_obj

COMPONENTS = ["IDComponent", "TagComponent", "RelationshipComponent", "TransformComponent",
              "SPHSimulationComponent", "MaterialComponent", "MeshComponent", "RigidBodyComponent",
              "FluidObjectComponent", "DFSPHSimulationComponent"]

# DFSPHSimulationDescription fields in the order of its serializer
# (Scene/Components/DFSPHSimulationComponent.h:7-39); the archive names are the field
# names with a lower-case first letter, except CSDFix and CSD.
_DESC_FIELDS = [name for name, _ in _abi.vfd_desc._fields_]
_NULL_ENTITY = 4294967295
_BOOL_FIELDS = ("EnableDivergenceSolverError", "EnableViscositySolver", "EnableSurfaceTensionSolver",
                "TemporalSmoothing")


def _archive_name(field: str) -> str:
    return field if field in ("CSDFix", "CSD") else field[0].lower() + field[1:]


def _xyz(d) -> list:
    return [d["x"], d["y"], d["z"]]


def _matrix(t) -> np.ndarray:
    cols = [t[f"value{j}"] for j in range(4)]
    return np.array([[c["x"], c["y"], c["z"], c["w"]] for c in cols], np.float32).T


def _unpack(doc: dict) -> list:
    vals, i = [], 0
    while f"value{i}" in doc:
        vals.append(doc[f"value{i}"])
        i += 1
    return vals


def load_scene(path: str) -> dict:
    """The entities, components, simulation description and scene data of a scene file."""
    with open(path, "r") as fh:
        doc = json.load(fh)
    vals = _unpack(doc)
    first = next((i for i, v in enumerate(vals) if isinstance(v, dict)), None)
    comps = {name: {} for name in COMPONENTS}
    entities = []
    if first is not None:
        if first < 2:
            raise ValueError(f"{path}: not an entity snapshot")
        start = first - 2
        entities = [int(v) for v in vals[2:start]]
        pos = start
        for name in COMPONENTS:
            if pos >= len(vals):
                raise ValueError(f"{path}: snapshot ends before {name}")
            count = int(vals[pos])
            pos += 1
            for _ in range(count):
                if pos + 1 >= len(vals):
                    raise ValueError(f"{path}: snapshot ends inside {name}")
                ent, payload = int(vals[pos]), vals[pos + 1]
                if not isinstance(payload, dict):
                    raise ValueError(f"{path}: malformed {name} entry at value{pos}")
                comps[name][ent] = payload
                pos += 2
        if pos != len(vals):
            raise ValueError(f"{path}: {len(vals) - pos} values after the last component")
    return dict(entities=entities, components=comps, scene_data=doc.get("sceneData", {}), path=path)


def description(scene: dict, entity: int | None = None) -> dict:
    """The DFSPH description (vfd_desc field names) of the scene's DFSPHSimulation component."""
    sims = scene["components"]["DFSPHSimulationComponent"]
    if not sims:
        raise ValueError("the scene has no DFSPH simulation component")
    src = sims[entity if entity is not None else sorted(sims)[0]]["description"]
    out = {}
    for f in _DESC_FIELDS:
        key = _archive_name(f)
        if key in src:
            v = src[key]
            out[f] = _xyz(v) if f == "Gravity" else (int(v) if isinstance(v, bool) else v)
    return out


def world_transform(scene: dict, entity: int) -> np.ndarray:
    """Scene::GetWorldSpaceTransformMatrix: parent world transform times the local one."""
    comps = scene["components"]
    by_uuid = {c["id"]["UUID32"]: e for e, c in comps["IDComponent"].items()}
    m = np.eye(4, dtype=np.float64)
    chain, e, seen = [], entity, set()
    while e is not None and e not in seen:
        seen.add(e)
        chain.append(e)
        rel = comps["RelationshipComponent"].get(e)
        parent = rel["parent"]["UUID32"] if rel else 0
        e = by_uuid.get(parent) if parent else None
    for e in reversed(chain):
        t = comps["TransformComponent"].get(e)
        if t is not None:
            m = m @ _matrix(t["transform"]).astype(np.float64)
    return m.astype(np.float32)


def _resolve(mesh_source: str, mesh_root: str | None, scene_path: str | None) -> str:
    if os.path.isabs(mesh_source):
        return mesh_source
    for base in (mesh_root, os.path.dirname(scene_path) if scene_path else None, os.getcwd()):
        if base and os.path.exists(os.path.join(base, mesh_source)):
            return os.path.join(base, mesh_source)
    raise FileNotFoundError(f"mesh {mesh_source!r} not found (mesh_root={mesh_root!r})")


def objects(scene: dict, mesh_root: str | None = None) -> dict:
    """Fluid objects and rigid bodies with their meshes loaded and world transforms."""
    comps = scene["components"]
    meshes_ = {}

    def mesh(e):
        src = comps["MeshComponent"][e]["meshSource"]
        if src not in meshes_:
            meshes_[src] = load_obj(_resolve(src, mesh_root, scene.get("path")))
        return meshes_[src]

    fluids, bodies = [], []
    for e in scene["entities"]:
        if e in comps["FluidObjectComponent"] and e in comps["MeshComponent"]:
            c = comps["FluidObjectComponent"][e]
            v, t = mesh(e)
            fluids.append(dict(entity=e, vertices=v, triangles=t, transform=world_transform(scene, e),
                               inverted=bool(c["inverted"]), resolution=_xyz(c["resolution"]),
                               sample_mode=int(c["sampleMode"]), velocity=_xyz(c["velocity"])))
        if e in comps["RigidBodyComponent"] and e in comps["MeshComponent"]:
            c = comps["RigidBodyComponent"][e]
            v, t = mesh(e)
            bodies.append(dict(entity=e, vertices=v, triangles=t, transform=world_transform(scene, e),
                               inverted=bool(c["inverted"]), padding=float(c["padding"]),
                               resolution=_xyz(c["collisionMapResolution"])))
    return dict(fluids=fluids, bodies=bodies)


def bake(scene: dict, mesh_root: str | None = None, desc_overrides: dict | None = None):
    """A DFSPHSimulation holding the scene's fluid objects and rigid bodies (Bake Objects),
    with the particles and maps made on the GPU. Returns (simulation, objects)."""
    from . import DFSPHSimulation, build_mesh_map, sample_mesh_volume
    d = description(scene)
    if desc_overrides:
        d.update(desc_overrides)
    sim = DFSPHSimulation(_abi.make_desc(**d))
    r = float(d.get("ParticleRadius", _abi.DEFAULTS["ParticleRadius"]))
    obj = objects(scene, mesh_root)
    xs, vs = [], []
    for f in obj["fluids"]:
        x = sample_mesh_volume(f["vertices"], f["triangles"], r, f["resolution"], f["inverted"], f["sample_mode"],
                               transform=f["transform"])
        f["particles"] = len(x)
        xs.append(x)
        vs.append(np.tile(np.asarray(f["velocity"], np.float32), (len(x), 1)))
    x = np.concatenate(xs) if xs else np.zeros((0, 3), np.float32)
    v = np.concatenate(vs) if vs else np.zeros((0, 3), np.float32)
    sim.SetFluidObjects(x, v)
    for b in obj["bodies"]:
        b["map"] = build_mesh_map(b["vertices"], b["triangles"], b["transform"], b["inverted"], b["padding"],
                                  b["resolution"], r)
        sim.AddRigidBody(b["map"])
    return sim, obj


# ---------------------------------------------------------------- writing
def _vec3(v) -> dict:
    return {"x": float(v[0]), "y": float(v[1]), "z": float(v[2])}


def _uvec3(v) -> dict:
    return {"x": int(v[0]), "y": int(v[1]), "z": int(v[2])}


def save_scene(path: str, entities: list, scene_data: dict | None = None) -> None:
    """Writes a scene file in the reference's layout. `entities` is a list of dicts with
    keys uuid, tag, transform (4x4), parent (uuid or 0) and optionally mesh (path),
    material (dict), rigid_body {inverted, padding, resolution}, fluid {inverted,
    resolution, sample_mode, velocity} and dfsph (a description dict, vfd_desc names)."""
    vals = [len(entities) + 1, _NULL_ENTITY] + list(range(len(entities)))

    def section(name, make):
        pairs = [(i, make(e)) for i, e in enumerate(entities) if make(e) is not None]
        vals.append(len(pairs))
        for i, payload in pairs:
            vals.extend([i, payload])

    def transform(e):
        m = np.asarray(e.get("transform", np.eye(4)), np.float32)
        return {"transform": {f"value{j}": {"x": float(m[0, j]), "y": float(m[1, j]), "z": float(m[2, j]),
                                             "w": float(m[3, j])} for j in range(4)}}

    def dfsph(e):
        if "dfsph" not in e:
            return None
        full = dict(_abi.DEFAULTS)
        full.update(e["dfsph"])
        desc = {}
        for f in _DESC_FIELDS:
            v = full[f]
            if f == "Gravity":
                v = _vec3(v)
            elif f in _BOOL_FIELDS:
                v = bool(v)
            desc[_archive_name(f)] = v
        return {"description": desc}

    section("IDComponent", lambda e: {"id": {"UUID32": int(e["uuid"])}})
    section("TagComponent", lambda e: {"tag": e.get("tag", "Entity")})
    section("RelationshipComponent",
            lambda e: {"parent": {"UUID32": int(e.get("parent", 0))},
                       "children": [{"UUID32": int(c["uuid"])} for c in entities
                                    if int(c.get("parent", 0)) == int(e["uuid"])]})
    section("TransformComponent", transform)
    section("SPHSimulationComponent", lambda e: e.get("sph"))
    section("MaterialComponent", lambda e: e.get("material"))
    section("MeshComponent", lambda e: {"meshSource": e["mesh"]} if "mesh" in e else None)
    section("RigidBodyComponent", lambda e: None if "rigid_body" not in e else {
        "inverted": bool(e["rigid_body"].get("inverted", False)),
        "padding": float(e["rigid_body"].get("padding", 0.0)),
        "collisionMapResolution": _uvec3(e["rigid_body"].get("resolution", (20, 20, 20)))})
    section("FluidObjectComponent", lambda e: None if "fluid" not in e else {
        "inverted": bool(e["fluid"].get("inverted", False)),
        "resolution": _uvec3(e["fluid"].get("resolution", (20, 20, 20))),
        "sampleMode": int(e["fluid"].get("sample_mode", 0)),
        "velocity": _vec3(e["fluid"].get("velocity", (0.0, 0.0, 0.0)))})
    section("DFSPHSimulationComponent", dfsph)
    doc = {f"value{i}": v for i, v in enumerate(vals)}
    doc["sceneData"] = scene_data if scene_data is not None else {
        "cameraPosition": _vec3((4.0, 4.0, 4.0)), "cameraPivot": _vec3((0.0, 0.0, 0.0)), "readMe": ""}
    with open(path, "w") as fh:
        json.dump(doc, fh, indent=4)


class FrameWriter:
    """Writes the frames of DFSPHSimulation.Simulate to `directory` (frame_NNNNN.npz with
    x, v, a as float32 (n, 3), plus index.json with per-frame time step and maximum
    speed). Use as the on_frame callback: sim.Simulate(FrameWriter(dir))."""

    def __init__(self, directory: str, fields=("x", "v", "a")):
        self.directory = directory
        self.fields = tuple(fields)
        self.index = []
        os.makedirs(directory, exist_ok=True)

    def __call__(self, idx, x, v, a, max_velocity, dt):
        data = {"x": x, "v": v, "a": a}
        name = f"frame_{idx:05d}.npz"
        np.savez(os.path.join(self.directory, name), **{k: data[k] for k in self.fields})
        self.index.append(dict(frame=int(idx), file=name, particles=int(len(x)), time_step=float(dt),
                               max_velocity=float(max_velocity)))
        with open(os.path.join(self.directory, "index.json"), "w") as fh:
            json.dump(self.index, fh, indent=1)


def read_frames(directory: str):
    """(index entries, loader) of a FrameWriter directory; loader(i) -> dict of arrays."""
    with open(os.path.join(directory, "index.json")) as fh:
        index = json.load(fh)

    def load(i):
        with np.load(os.path.join(directory, index[i]["file"])) as z:
            return {k: z[k] for k in z.files}

    return index, load
