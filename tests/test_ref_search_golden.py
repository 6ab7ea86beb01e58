"""The oracle's neighbour search against the reference's own search kernels.

tests/golden/ref_search.json holds SHA-256 digests of what the reference's
ParticleSearchKernels.cu computes (compiled for the CPU with a CUDA/glm stand-in and
run one emulated thread at a time, so its atomic in-cell ranks come out in ascending
particle index) on four seeded inputs: the 8,000-particle dam break, the 64,000-particle
viscous dam break, dense cells with particles past the 70-neighbour cap, and a uniform
cloud with negative coordinates. The FP32 oracle must reproduce every output bit for
bit: counts, offsets, the CSR list (original indices, z-y-x cell order), the sort
permutation and the Morton meta-grid cell keys. The GPU search is held to the same
digests in tests/test_gpu_parity.py."""
import hashlib
import json
import os
import sys

import numpy as np
import pytest

from oracle import oracle as O
from vfd_gb300 import _abi

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_ref_search as M  # noqa: E402

GOLDEN = json.load(open(os.path.join(HERE, "golden", "ref_search.json")))


def digests(r: dict) -> dict:
    return {k: hashlib.sha256(np.ascontiguousarray(v, np.uint32).tobytes()).hexdigest() for k, v in r.items()}


@pytest.mark.parametrize("name", sorted(GOLDEN["cases"]))
def test_oracle_search_equals_reference_kernels(name):
    x, h = M.cases()[name]
    ref = GOLDEN["cases"][name]
    assert len(x) == ref["n"] and h == pytest.approx(ref["h"])
    o = O.OracleSim(_abi.make_desc(ParticleRadius=h / 4), 32)
    o.set_fluid(x, None)
    o.find_neighbors()
    b = o.neighbors()
    assert digests(b) == ref["sha256"]
    for i, row in ref["rows"].items():
        i = int(i)
        assert b["list"][b["offsets"][i]:b["offsets"][i] + b["counts"][i]].tolist() == row


@pytest.mark.skipif(not os.path.exists(M.LIB), reason="the reference's search kernels are built only where its "
                                                      "sources are (oracle/Makefile target ref)")
@pytest.mark.parametrize("name", ["dam_break_8k", "dense_cells_and_cap"])
def test_reference_search_library_reproduces_the_fixture(name):
    """The committed digests are what the compiled reference kernels compute: rerun."""
    x, h = M.cases()[name]
    r = M.run_reference(x, h)
    assert {k: M.digest(v) for k, v in r.items()} == GOLDEN["cases"][name]["sha256"]
