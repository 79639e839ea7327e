"""Multi-rank host logic on CPU ranks (gloo, world_size 2): the sharding of
independent systems by vertex count and the whole-job reduction bench.py
applies to replicas (slowest rank's time, sum of pair evaluations)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from pycudapolygon_gb300.systems import batched_specs, shard_by_vertices  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        specs = batched_specs(16, seed=3)
        counts = [int(sum(n)) for (_, n, _, _) in specs]
        mine = shard_by_vertices(counts, world)[rank]
        # every rank computes the same assignment without communicating
        gathered = [None] * world
        dist.all_gather_object(gathered, mine)
        # a replica's timed region: rank-dependent time and pair count
        ms, pairs = bench.reduce_over_ranks(10.0 + rank, 100 * (rank + 1), dist, "cpu")
        out[rank] = (gathered, ms, pairs, sum(counts[i] for i in mine))
    finally:
        dist.destroy_process_group()


def test_sharding_and_replica_reduction_on_two_gloo_ranks():
    world = 2
    manager = mp.Manager()
    out = manager.dict()
    mp.spawn(_worker, args=(world, _free_port(), out), nprocs=world, join=True)
    g0, ms0, p0, load0 = out[0]
    g1, ms1, p1, load1 = out[1]
    assert g0 == g1                                   # same plan on every rank
    shards = g0
    assert sorted(shards[0] + shards[1]) == list(range(16))
    assert not set(shards[0]) & set(shards[1])
    assert (ms0, p0) == (ms1, p1) == (11.0, 300.0)    # max time, summed pairs
    assert abs(load0 - load1) <= max(load0, load1) * 0.1


def test_shard_by_vertices_balances_and_is_deterministic():
    counts = [5, 1, 9, 3, 3, 7, 2, 8]
    s3 = shard_by_vertices(counts, 3)
    assert sorted(i for sh in s3 for i in sh) == list(range(len(counts)))
    loads = [sum(counts[i] for i in sh) for sh in s3]
    assert max(loads) - min(loads) <= max(counts)
    assert s3 == shard_by_vertices(counts, 3)
    assert shard_by_vertices(counts, 1) == [list(range(len(counts)))]
    assert shard_by_vertices([], 2) == [[], []]
