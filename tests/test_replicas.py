"""Multi-rank path of bench.py on CPU: two gloo ranks, each timing its own
replica, agree on the slowest rank's time and the whole-job throughput."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from saq_gb300.replicas import max_over_ranks, replica_throughput
    my = 1.0 + rank  # rank 1 is the slow one
    out[rank] = (max_over_ranks(my, "cpu"), replica_throughput(4096, my, world, "cpu"))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2])
def test_two_gloo_ranks_take_the_slowest(world):
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    assert res[0] == res[1] == (2.0, 2 * 4096 / 2.0)


def test_single_process_is_its_own_max():
    from saq_gb300.replicas import max_over_ranks, replica_throughput
    assert not dist.is_initialized()
    assert max_over_ranks(3.5, "cpu") == 3.5
    assert replica_throughput(100, 2.0, 1, "cpu") == 50.0
