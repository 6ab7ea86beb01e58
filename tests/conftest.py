"""Test configuration: the `gpu` marker and shared fixtures.

Tests marked `gpu` need a CUDA device and call the library through its C-ABI;
the others run on the CPU (oracle against golden data, host logic, library
loading and exports).
"""
import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); calls the CUDA library")


@pytest.fixture(scope="session")
def golden():
    with open(os.path.join(ROOT, "tests", "golden", "reference_tables.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def built_library():
    """The CUDA library, compiled if needed (nvcc cross-compiles without a GPU)."""
    from vfd_gb300 import build
    return build.build()
