"""The bounds-checked build on a parity scene: no device index check fails, and the
results equal the release build's bit for bit (the checks change no arithmetic).
The checked library runs in a child process (a process loads one build)."""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import sys, numpy as np
sys.path.insert(0, sys.argv[1])
import vfd_gb300 as V
from vfd_gb300 import scenes
s = scenes.small_dam_break(n_side=10, viscosity=0.02, surface_tension=0.05)
sim = V.scene_simulation(s)
st = sim.Steps(5)
x, v, _ = sim.GetState()
np.savez(sys.argv[2], x=x, v=v, flags=st["Flags"])
"""


def run_child(tmp_path, library, tag):
    out = str(tmp_path / f"{tag}.npz")
    env = dict(os.environ, VFD_LIBRARY=library)
    r = subprocess.run([sys.executable, "-c", CHILD, ROOT, out], env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return np.load(out)


def test_bounds_checked_build_matches_release(tmp_path):
    from vfd_gb300 import build
    checked = build.build(bounds_check=True)
    release = build.build()
    a = run_child(tmp_path, checked, "checked")
    b = run_child(tmp_path, release, "release")
    assert int(a["flags"]) & 0x80 == 0
    np.testing.assert_array_equal(a["x"], b["x"])
    np.testing.assert_array_equal(a["v"], b["v"])
