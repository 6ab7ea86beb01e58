"""Scene baking and headless frames on the GPU: the authored fixture
tests/golden/scenes/drop.json is baked (its fluid sphere sampled by
vfd_sample_mesh_volume, its container mapped by vfd_build_mesh_map, both placed by
their world transforms), the particles equal the oracle's ParticleSampler of the same
placed mesh, the map equals the oracle's mesh map within the FP32 error of the
reference's distance, and Simulate writes FrameCount frames that read back."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from vfd_gb300 import scene_io

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "golden", "scenes", "drop.json")


def test_bake_and_simulate(tmp_path):
    scene = scene_io.load_scene(FIXTURE)
    sim, obj = scene_io.bake(scene)
    f, b = obj["fluids"][0], obj["bodies"][0]
    r = scene_io.description(scene)["ParticleRadius"]
    x0, v0, _ = sim.GetState()
    ref = O.sample_mesh_volume(f["vertices"], f["triangles"], r, f["resolution"], f["inverted"], f["sample_mode"],
                               transform=f["transform"])
    assert sim.GetParticleCount() == len(x0) == f["particles"]
    sa, sb = {tuple(p) for p in x0.tolist()}, {tuple(p) for p in ref.tolist()}
    print(f"{len(x0)} particles baked, oracle {len(ref)}, {len(sa ^ sb)} differ")
    assert len(sa ^ sb) <= 2 + 1e-3 * len(ref)
    np.testing.assert_array_equal(v0, np.tile(np.float32([0.5, 0.0, 0.0]), (len(x0), 1)))
    assert np.all(np.abs(np.linalg.norm(x0 - [0.3, 0.4, 0.3], axis=1)) < 0.15 + 1e-3)
    m = O.build_mesh_map(b["vertices"], b["triangles"], b["transform"], b["inverted"], b["padding"],
                         b["resolution"], r)
    nn = m.struct.node_count
    assert b["map"].meta() == m.meta()
    assert np.abs(b["map"].nodes[:nn] - m.nodes[:nn]).max() < 1e-4

    writer = scene_io.FrameWriter(str(tmp_path / "frames"))
    frames = sim.Simulate(writer)
    assert frames == 3
    index, load = scene_io.read_frames(str(tmp_path / "frames"))
    assert [e["frame"] for e in index] == [0, 1, 2]
    last = load(2)
    assert last["x"].shape == x0.shape and np.all(np.isfinite(last["x"]))
    assert np.all(last["x"] > -1e-3) and np.all(last["x"] < np.array([1.2, 0.8, 0.6]) + 1e-3)
    assert last["x"][:, 0].mean() > x0[:, 0].mean()  # the drop moves with its initial velocity
