"""Golden neighbour searches from the reference's own search kernels.

Builds oracle/_ref/libvfd_refsearch.so (the reference's
Simulation/DFSPH/ParticleSearch/ParticleSearchKernels.cu compiled for the CPU with a
CUDA/glm stand-in header, beside a restatement of its host driver; recipe in
oracle/Makefile, target `ref`), runs it on seeded inputs and writes
tests/golden/ref_search.json: for each case its inputs' recipe, the particle count and
SHA-256 digests of the five outputs (neighbour counts, offsets, the CSR list of original
indices, the sort permutation, the cell keys), plus a few rows for reading. The
reference's in-cell order comes from atomicAdd ranks; the emulated threads run in
particle order, which gives ascending original index, the order the oracle and the CUDA
library use, so the digests compare bit for bit.

Usage: python tests/golden/make_ref_search.py VFD_ROOT
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from vfd_gb300 import scenes  # noqa: E402

LIB = os.path.join(ROOT, "oracle", "_ref", "libvfd_refsearch.so")


def cases() -> dict:
    """Seeded inputs (positions, search radius h) rebuilt identically by the tests."""
    out = {}
    s = scenes.dam_break_8k()
    out["dam_break_8k"] = (s["x"], 4 * s["desc"]["ParticleRadius"])
    s = scenes.viscous_dam_break(n_side=40)
    out["viscous_dam_break_64k"] = (s["x"], 4 * s["desc"]["ParticleRadius"])
    out["dense_cells_and_cap"] = dense_case()
    out["uniform_cloud_20k"] = uniform_cloud()
    return out


def dense_case():
    """A small dam break plus a blob of 3000 particles in a 2.5 h cube: cells of 100+
    particles and particles past the 70-neighbour cap."""
    s = scenes.small_dam_break(n_side=8)
    h = 4 * s["desc"]["ParticleRadius"]
    rng = np.random.default_rng(3000)
    blob = (np.float32([0.6, 0.3, 0.3]) + 2.5 * h * rng.random((3000, 3))).astype(np.float32)
    return np.concatenate([s["x"], blob]).astype(np.float32), h


def uniform_cloud():
    """20,000 particles uniform in a 1 x 0.5 x 0.7 m box, h = 0.05 (sparse and dense cells,
    negative coordinates)."""
    u = scenes.SplitMix64(20000).uniform(60000).reshape(-1, 3)
    x = (u * np.array([1.0, 0.5, 0.7]) - np.array([0.3, 0.1, 0.2])).astype(np.float32)
    return x, 0.05


def run_reference(x: np.ndarray, h: float) -> dict:
    lib = C.CDLL(LIB)
    f = lib.ref_find_neighbors
    u32p = C.POINTER(C.c_uint32)
    f.argtypes = [C.POINTER(C.c_float), C.c_uint32, C.c_float, u32p, u32p, u32p, C.c_uint32, u32p, u32p, u32p]
    f.restype = C.c_int
    x = np.ascontiguousarray(x, np.float32)
    n = len(x)
    counts, offsets, sort_idx, keys = (np.zeros(n, np.uint32) for _ in range(4))
    total = C.c_uint32()
    P = lambda a: a.ctypes.data_as(u32p)  # noqa: E731
    rc = f(x.ctypes.data_as(C.POINTER(C.c_float)), n, h, P(counts), P(offsets), None, 0, C.byref(total),
           P(sort_idx), P(keys))
    assert rc == 0, rc
    lst = np.zeros(max(1, total.value), np.uint32)
    rc = f(x.ctypes.data_as(C.POINTER(C.c_float)), n, h, None, None, P(lst), total.value, C.byref(total), None, None)
    assert rc == 0, rc
    return dict(counts=counts, offsets=offsets, list=lst[:total.value], sort_indices=sort_idx, cell_keys=keys)


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, np.uint32).tobytes()).hexdigest()


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_ref_search.py VFD_ROOT")
    subprocess.run(["make", "-s", "ref", f"REF={sys.argv[1]}"], cwd=os.path.join(ROOT, "oracle"), check=True)
    out = {"source": "VFD ParticleSearchKernels.cu run on the CPU (oracle/ref_search, oracle/Makefile target ref)",
           "cases": {}}
    for name, (x, h) in cases().items():
        r = run_reference(x, h)
        out["cases"][name] = {
            "n": int(len(x)), "h": float(h), "total": int(len(r["list"])), "max_count": int(r["counts"].max()),
            "sha256": {k: digest(v) for k, v in r.items()},
            "rows": {str(i): r["list"][r["offsets"][i]:r["offsets"][i] + r["counts"][i]].tolist()
                     for i in (0, len(x) // 2, len(x) - 1)},
        }
        print(name, len(x), "particles,", len(r["list"]), "pairs, max count", int(r["counts"].max()))
    with open(os.path.join(HERE, "ref_search.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
