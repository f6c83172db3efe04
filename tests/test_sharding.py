"""Scene-parallel sharding of batches (host logic, no GPU): the partition of scenes
over ranks, and the two collectives on two gloo ranks. These are the sum of
shared-parameter gradients and the whole-job rate."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from mpm_engine_gb300.scenes import squeeze_batch_specs
from mpm_engine_gb300.sharding import imbalance, partition, reduce_shared_gradients, sharded_throughput


def test_partition_covers_each_scene_once_and_balances():
    counts = [sp["n_particles"] for sp in squeeze_batch_specs(64)]
    for world in (1, 2, 3, 4, 8):
        parts = partition(counts, world)
        assert len(parts) == world
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(64))
        assert all(p == sorted(p) for p in parts)
        assert imbalance(parts, counts) < 1.05, (world, imbalance(parts, counts))
        assert partition(counts, world) == parts          # every rank computes the same split


def test_partition_edge_cases():
    assert partition([], 3) == [[], [], []]
    assert partition([5.0, 1.0], 4) == [[0], [1], [], []]
    assert partition([1.0, 1.0, 1.0, 1.0], 2) == [[0, 2], [1, 3]]
    with pytest.raises(ValueError):
        partition([1.0], 0)
    assert imbalance([[0], []], [2.0]) == pytest.approx(2.0)


def test_single_process_collectives_are_local():
    g = {"E": torch.tensor([1.5]), "nu": torch.tensor([-2.0])}
    assert reduce_shared_gradients(g) is g and g["E"].item() == 1.5
    rate, units, sec = sharded_throughput(100.0, 0.5)
    assert (rate, units, sec) == (200.0, 100.0, 0.5)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    counts = [sp["n_particles"] for sp in squeeze_batch_specs(16)]
    mine = partition(counts, world)[rank]
    # per-scene gradients of shared parameters, summed locally, then over the ranks
    local = {"E": torch.tensor([float(sum(mine))], dtype=torch.float64),
             "nu": torch.tensor([float(len(mine))], dtype=torch.float64)}
    reduce_shared_gradients(local)
    units = float(sum(counts[i] for i in mine))
    rate, total, sec = sharded_throughput(units, 1.0 + rank)
    out[rank] = (local["E"].item(), local["nu"].item(), rate, total, sec, mine)
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_shard_and_reduce():
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    counts = [sp["n_particles"] for sp in squeeze_batch_specs(16)]
    assert sorted(res[0][5] + res[1][5]) == list(range(16))
    for r in range(2):
        e, nu, rate, total, sec, _ = res[r]
        assert e == pytest.approx(sum(range(16)))         # every scene's contribution, once
        assert nu == pytest.approx(16)
        assert total == pytest.approx(float(np.sum(counts)))
        assert sec == pytest.approx(2.0)                  # the slower rank's time
        assert rate == pytest.approx(float(np.sum(counts)) / 2.0)
