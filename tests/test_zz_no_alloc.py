"""The allocation-free neighbour search against the regular entry point.

vfd_find_neighbors_noalloc serves callers that cannot allocate device memory
(their memory belongs to another allocator with a fixed budget, or they must not
allocate once running): the caller brings device buffers for positions and
results, and the search keeps its intermediate data in a fixed internal device
array. Here the caller's buffers come from torch; the results of two calls in a
row (different particle sets, the second overwriting what the first left in the
shared array) must equal the regular search's exactly (integer outputs).
This file is collected last on purpose.
"""
import numpy as np
import pytest

import vfd_gb300 as V
from vfd_gb300 import _abi, scenes

pytestmark = pytest.mark.gpu


def regular_search(x, r):
    sim = V.DFSPHSimulation(_abi.make_desc(ParticleRadius=r))
    sim.SetFluidObjects(x)
    sim.FindNeighbors()
    return sim.GetNeighbors()


def noalloc_search(x, r):
    import torch
    n = len(x)
    xyz = torch.from_numpy(np.ascontiguousarray(x, np.float32)).cuda()
    counts = torch.zeros(n, dtype=torch.int32, device="cuda")
    rows = torch.full((n, _abi.MAX_NEIGHBORS), -1, dtype=torch.int32, device="cuda")
    sort_idx = torch.zeros(n, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    rc = V.find_neighbors_noalloc(xyz.data_ptr(), n, r, counts.data_ptr(), rows.data_ptr(), sort_idx.data_ptr())
    torch.cuda.synchronize()
    return rc, counts.cpu().numpy().astype(np.uint32), rows.cpu().numpy().astype(np.uint32), \
        sort_idx.cpu().numpy().astype(np.uint32)


def check_equal(x, r):
    ref = regular_search(x, r)
    rc, counts, rows, sort_idx = noalloc_search(x, r)
    assert rc == _abi.VFD_OK
    np.testing.assert_array_equal(counts, ref["counts"])
    np.testing.assert_array_equal(sort_idx, ref["sort_indices"])
    flat = np.concatenate([rows[i, :counts[i]] for i in range(len(x))]) if len(x) else np.zeros(0, np.uint32)
    np.testing.assert_array_equal(flat, ref["list"])


def test_noalloc_search_matches_regular_search_twice():
    a = scenes.dam_break_8k()                      # 8000 particles, r = 0.025
    b = scenes.small_dam_break(n_side=14, seed=3)  # 2744 particles, other positions
    check_equal(a["x"], a["desc"]["ParticleRadius"])
    check_equal(b["x"], b["desc"]["ParticleRadius"])


def test_noalloc_search_rejects_too_many_particles():
    x = scenes.lattice_block((26, 26, 26), 0.01, (0, 0, 0), 0.05, scenes.SplitMix64(1))  # 17576 > 16384
    rc, _, _, _ = noalloc_search(x, 0.01)
    assert rc == _abi.VFD_E_CAPACITY


def test_noalloc_search_device_side_rejections_leave_it_usable():
    """Rejections found on the device come back as status codes, and a call after
    them (the abort flags and buckets live in the shared array) is still exact."""
    r = 0.01
    far = np.float32([[0.0, 0.0, 0.0], [1000.0, 0.0, 0.0]])  # a grid of ~1.6M cells > 262144
    rc, _, _, _ = noalloc_search(far, r)
    assert rc == _abi.VFD_E_CAPACITY
    x = scenes.lattice_block((6, 6, 6), r, (0, 0, 0), 0.05, scenes.SplitMix64(2))
    bad = x.copy()
    bad[17, 2] = np.nan
    rc, _, _, _ = noalloc_search(bad, r)
    assert rc == _abi.VFD_E_NAN
    check_equal(x, r)
