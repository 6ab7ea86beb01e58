"""The bounds-checked build (-DVFD_BOUNDS_CHECK) compiles and exports the same
entry points. Its device checks record failures in the status word instead of
faulting; the GPU test (test_gpu_bounds_check.py) runs it on a parity scene."""
import ctypes

import vfd_gb300
from vfd_gb300 import build


def test_bounds_checked_library_builds_and_exports_everything():
    path = build.build(bounds_check=True)
    lib = ctypes.CDLL(path)
    for name in vfd_gb300.EXPORTS:
        assert hasattr(lib, name), name
