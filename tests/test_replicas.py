"""Replica scaling of bench.py on CPU: two gloo ranks, each timing its own replica;
the whole-job value is every rank's work over the slowest rank's time."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    local_ms = 100.0 * (rank + 1)          # rank 1 is the slow replica
    value, ms = bench.replica_value(local_ms, units_per_step=1000.0, steps=4, world=world, dist=dist)
    out[rank] = (value, ms)
    dist.barrier()
    dist.destroy_process_group()


def test_replica_value_takes_the_slowest_rank():
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
    for r in range(2):
        value, ms = res[r]
        assert ms == pytest.approx(200.0)
        assert value == pytest.approx(2 * 1000.0 * 4 / 0.2)


def test_single_rank_value_is_its_own():
    import bench
    value, ms = bench.replica_value(50.0, units_per_step=10.0, steps=2, world=1)
    assert ms == 50.0 and value == pytest.approx(10.0 * 2 / 0.05)


def test_bench_reads_its_committed_profile_figures():
    """The roofline's DRAM traffic and the press's FLOP count come from the ncu
    summaries under profiles/: a renamed file or line would leave them null."""
    import bench
    assert bench.captured_traffic("pour_honey_192^3") > 0
    assert bench.captured_traffic("pour_honey_cdf_glasses_192^3") > 0
    flops = bench.captured_value("particle_passes_press_mu_i_256.txt", "fp32_flops_per_particle_substep")
    assert flops is not None and 1000 < flops < 10000
