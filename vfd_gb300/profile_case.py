"""Runs one configuration of the DFSPH step for a profiler (ncu) to capture.

python -m vfd_gb300.profile_case [n_side] [lanes]

Builds the viscous dam break of n_side^3 particles (BASELINE config 2 parameters),
takes `graph_steps` steps as one CUDA graph each (lanes per particle: 4, 8, 16, or 0 =
autotune), then `eager_steps` steps with every kernel launched from the host, so that a
profiler filtering by kernel name sees individual launches of every kernel.
"""
from __future__ import annotations

import sys

from . import TUNED_KERNELS, scene_simulation
from . import scenes


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    n_side = int(argv[0]) if len(argv) > 0 else 80
    lanes = int(argv[1]) if len(argv) > 1 else 0
    graph_steps = int(argv[2]) if len(argv) > 2 else 4
    eager_steps = int(argv[3]) if len(argv) > 3 else 2
    s = scenes.viscous_dam_break(n_side=n_side)
    sim = scene_simulation(s)
    sim.Steps(2)
    if lanes:
        sim.SetLanes([lanes] * len(TUNED_KERNELS))
    else:
        print("lanes", sim.Autotune(1))
    sim.Steps(graph_steps)
    sim.SetGraphMode(False)
    st = sim.Steps(eager_steps)
    print("particles", len(s["x"]), "stats", st)


if __name__ == "__main__":
    main()
