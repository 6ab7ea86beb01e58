"""Batches across ranks (vfd_gb300.partition): the scene assignment and the host-side
gather of per-scene statistics, with two gloo ranks on the CPU."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from vfd_gb300 import partition, scenes


def test_every_scene_is_assigned_once_and_balanced():
    costs = [len(s["x"]) for s in scenes.uneven_batch()]
    for world in (1, 2, 4, 8):
        parts = partition.assign(costs, world)
        assert sorted(i for p in parts for i in p) == list(range(len(costs)))
        assert partition.imbalance(costs, parts) < 1.01
    assert partition.assign(costs, 4) == partition.assign(costs, 4)


def test_largest_scenes_go_to_different_ranks():
    parts = partition.assign([100, 90, 10, 5, 1], 2)
    assert {0, 1} != set(parts[0]) and {0, 1} != set(parts[1])


def test_edge_cases():
    # more ranks than scenes: some ranks get none; no scenes: every rank gets none
    parts = partition.assign([5, 3], 4)
    assert sorted(i for p in parts for i in p) == [0, 1] and sum(1 for p in parts if not p) == 2
    assert partition.assign([], 3) == [[], [], []]
    assert partition.imbalance([], [[], []]) == 1.0
    # equal costs split evenly, ties broken by index
    assert partition.assign([1] * 6, 3) == [[0, 3], [1, 4], [2, 5]]
    with pytest.raises(ValueError):
        partition.assign([1, 2], 0)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    rng = np.random.default_rng(1)
    batch = [dict(x=np.zeros((int(n), 3), np.float32)) for n in rng.integers(2000, 64000, 40)]
    idx, local = partition.local_scenes(batch, rank, world)
    stats = [{"particles": len(s["x"]), "rank": rank} for s in local]
    allstats = partition.gather_scene_stats(idx, stats, world)
    q.put((rank, sorted(allstats), {k: v["particles"] for k, v in allstats.items()}))
    dist.destroy_process_group()


def test_two_ranks_cover_the_batch_and_gather_its_statistics():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    rng = np.random.default_rng(1)
    sizes = [int(n) for n in rng.integers(2000, 64000, 40)]
    for rank, keys, parts in out:
        assert keys == list(range(40))
        assert [parts[k] for k in keys] == sizes
