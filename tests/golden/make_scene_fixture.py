"""Writes the scene fixture used by the scene-file tests: tests/golden/scenes/drop.json
and the meshes it names (scenes/Models/Box.obj, scenes/Models/Sphere.obj).

The scene is authored here (no reference file is copied): a DFSPH simulation entity, an
inverted box container scaled to 1.2 x 0.8 x 0.6 m, an empty "Group" entity translated
by (0.3, 0.2, 0.3) and, as its child, a sphere of radius 0.15 m sampled as fluid in
the densest packing with an initial velocity, in the layout the reference's
Scene::Save writes.

Usage: python tests/golden/make_scene_fixture.py
"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from vfd_gb300 import meshes, scene_io  # noqa: E402


def main():
    out = os.path.join(HERE, "scenes")
    os.makedirs(os.path.join(out, "Models"), exist_ok=True)
    meshes.save_obj(os.path.join(out, "Models", "Box.obj"), *meshes.box_mesh((-0.5, -0.5, -0.5), (0.5, 0.5, 0.5)))
    meshes.save_obj(os.path.join(out, "Models", "Sphere.obj"), *meshes.icosphere((0, 0, 0), 0.5, 2))
    desc = dict(ParticleRadius=0.02, TimeStepSize=0.001, MinTimeStepSize=0.0001, MaxTimeStepSize=0.005,
                FrameLength=0.01, FrameCount=3, MinPressureSolverIterations=2, MaxPressureSolverIterations=100,
                MaxPressureSolverError=10.0, EnableDivergenceSolverError=1, MinDivergenceSolverIterations=2,
                MaxDivergenceSolverIterations=100, MaxDivergenceSolverError=10.0, EnableViscositySolver=1,
                MaxViscositySolverError=0.1, Viscosity=0.5, BoundaryViscosity=0.5, EnableSurfaceTensionSolver=0,
                Gravity=(0.0, -9.81, 0.0))
    entities = [
        dict(uuid=1001, tag="GPU Simulation", dfsph=desc),
        dict(uuid=1002, tag="Container", mesh="Models/Box.obj",
             transform=meshes.transform((0.6, 0.4, 0.3), (1.2, 0.8, 0.6)),
             material={"shaderSource": "none", "properties": []},
             rigid_body=dict(inverted=True, padding=0.0, resolution=(24, 16, 12))),
        dict(uuid=1003, tag="Group", transform=meshes.transform((0.3, 0.2, 0.3))),
        dict(uuid=1004, tag="Drop", parent=1003, mesh="Models/Sphere.obj",
             transform=meshes.transform((0.0, 0.2, 0.0), (0.3, 0.3, 0.3), (0.0, 30.0, 0.0)),
             fluid=dict(inverted=False, resolution=(16, 16, 16), sample_mode=2, velocity=(0.5, 0.0, 0.0))),
    ]
    scene_io.save_scene(os.path.join(out, "drop.json"), entities)
    print("wrote", out)


if __name__ == "__main__":
    main()
