"""Scene files (CPU): the layout the loader assumes is the one pinned from the reference's
serializers (tests/golden/reference_tables.json, scene_format), the authored fixture
tests/golden/scenes/drop.json loads into the expected objects, scenes round-trip
through save_scene, and the frame writer's files read back.

Set VFD_REFERENCE_SCENE to a scene file saved by the reference to also parse it."""
import json
import os

import numpy as np
import pytest

from vfd_gb300 import _abi, meshes, scene_io

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "golden", "scenes", "drop.json")


def _golden():
    with open(os.path.join(HERE, "golden", "reference_tables.json")) as f:
        return json.load(f)["scene_format"]


def test_layout_matches_the_reference_serializers():
    g = _golden()
    assert scene_io.COMPONENTS == g["components"]
    names = [scene_io._archive_name(f) for f, _ in _abi.vfd_desc._fields_]
    assert names == g["dfsph_description"][:len(names)]
    assert g["rigid_body"] == ["inverted", "padding", "collisionMapResolution"]
    assert g["fluid_object"] == ["inverted", "resolution", "sampleMode", "velocity"]
    assert g["transform"][0] == "transform" and g["mesh"][0] == "meshSource"


def test_fixture_loads():
    s = scene_io.load_scene(FIXTURE)
    assert s["entities"] == [0, 1, 2, 3]
    tags = [s["components"]["TagComponent"][e]["tag"] for e in s["entities"]]
    assert tags == ["GPU Simulation", "Container", "Group", "Drop"]
    d = scene_io.description(s)
    assert d["ParticleRadius"] == pytest.approx(0.02) and d["FrameCount"] == 3
    assert d["EnableViscositySolver"] == 1 and d["EnableSurfaceTensionSolver"] == 0
    assert d["Gravity"] == pytest.approx([0.0, -9.81, 0.0])
    _abi.make_desc(**d)  # every field is a description field
    # the drop's world transform is the group's translation times its own placement
    w = scene_io.world_transform(s, 3)
    np.testing.assert_allclose(w, meshes.transform((0.3, 0.2, 0.3)) @
                               meshes.transform((0.0, 0.2, 0.0), (0.3, 0.3, 0.3), (0.0, 30.0, 0.0)), atol=1e-6)
    obj = scene_io.objects(s)
    assert len(obj["fluids"]) == 1 and len(obj["bodies"]) == 1
    f, b = obj["fluids"][0], obj["bodies"][0]
    assert f["sample_mode"] == 2 and f["velocity"] == [0.5, 0.0, 0.0] and f["resolution"] == [16, 16, 16]
    assert b["inverted"] and b["resolution"] == [24, 16, 12] and len(b["triangles"]) == 12
    placed = b["vertices"].astype(np.float64) @ b["transform"][:3, :3].T + b["transform"][:3, 3]
    np.testing.assert_allclose(placed.min(0), [0, 0, 0], atol=1e-6)
    np.testing.assert_allclose(placed.max(0), [1.2, 0.8, 0.6], atol=1e-6)
    c = f["vertices"].astype(np.float64) @ f["transform"][:3, :3].T + f["transform"][:3, 3]
    np.testing.assert_allclose(np.linalg.norm(c - [0.3, 0.4, 0.3], axis=1), 0.15, atol=1e-6)


def test_round_trip(tmp_path):
    s = scene_io.load_scene(FIXTURE)
    comps = s["components"]
    ents = []
    for e in s["entities"]:
        rel = comps["RelationshipComponent"][e]
        ent = dict(uuid=comps["IDComponent"][e]["id"]["UUID32"], tag=comps["TagComponent"][e]["tag"],
                   parent=rel["parent"]["UUID32"],
                   transform=scene_io._matrix(comps["TransformComponent"][e]["transform"]))
        if e in comps["MeshComponent"]:
            ent["mesh"] = comps["MeshComponent"][e]["meshSource"]
        if e in comps["MaterialComponent"]:
            ent["material"] = comps["MaterialComponent"][e]
        if e in comps["RigidBodyComponent"]:
            c = comps["RigidBodyComponent"][e]
            ent["rigid_body"] = dict(inverted=c["inverted"], padding=c["padding"],
                                     resolution=scene_io._xyz(c["collisionMapResolution"]))
        if e in comps["FluidObjectComponent"]:
            c = comps["FluidObjectComponent"][e]
            ent["fluid"] = dict(inverted=c["inverted"], resolution=scene_io._xyz(c["resolution"]),
                                sample_mode=c["sampleMode"], velocity=scene_io._xyz(c["velocity"]))
        if e in comps["DFSPHSimulationComponent"]:
            ent["dfsph"] = scene_io.description(s, e)
        ents.append(ent)
    out = tmp_path / "copy.json"
    scene_io.save_scene(str(out), ents, s["scene_data"])
    with open(FIXTURE) as f1, open(out) as f2:
        a, b = json.load(f1), json.load(f2)
    assert a.keys() == b.keys()
    for k in a:
        assert json.dumps(a[k], sort_keys=True) == json.dumps(b[k], sort_keys=True), k


def test_malformed_scenes_are_rejected(tmp_path):
    with open(FIXTURE) as f:
        doc = json.load(f)
    last = max(int(k[5:]) for k in doc if k.startswith("value"))
    del doc[f"value{last}"]  # the description payload
    p = tmp_path / "bad.json"
    p.write_text(json.dumps(doc))
    with pytest.raises(ValueError):
        scene_io.load_scene(str(p))
    s = scene_io.load_scene(FIXTURE)
    with pytest.raises(FileNotFoundError):
        scene_io.objects(dict(s, path=str(tmp_path / "elsewhere.json")), mesh_root=str(tmp_path / "none"))


def test_frame_writer(tmp_path):
    w = scene_io.FrameWriter(str(tmp_path / "frames"))
    rng = np.random.default_rng(0)
    data = [rng.standard_normal((50, 3)).astype(np.float32) for _ in range(6)]
    for i in range(2):
        w(i, data[3 * i], data[3 * i + 1], data[3 * i + 2], 1.5 + i, 0.001)
    index, load = scene_io.read_frames(str(tmp_path / "frames"))
    assert [e["frame"] for e in index] == [0, 1] and index[1]["max_velocity"] == 2.5
    np.testing.assert_array_equal(load(1)["v"], data[4])


@pytest.mark.skipif(not os.environ.get("VFD_REFERENCE_SCENE"), reason="no reference scene file given")
def test_reference_scene_parses():
    s = scene_io.load_scene(os.environ["VFD_REFERENCE_SCENE"])
    d = scene_io.description(s)
    _abi.make_desc(**d)
    assert s["components"]["DFSPHSimulationComponent"] and s["entities"]
    for e in s["components"]["TransformComponent"]:
        assert np.all(np.isfinite(scene_io.world_transform(s, e)))
