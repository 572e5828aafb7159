"""The bench's replica mode (one independent solve stream per rank, no
data-path collective): timings are the maximum over ranks and the job rate
counts every rank's solves.  Two gloo ranks on the CPU."""
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


def _rank_main(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        mine = [100.0 * (rank + 1), 50.0 + rank, 7.0 - rank]
        got = bench.max_over_ranks(mine, world, torch.device("cpu"))
        q.put((rank, got, bench.job_rate(world, 10, got[0])))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_job_rate_two_ranks():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, got, rate in res:
        assert got == [200.0, 51.0, 7.0]
        assert rate == pytest.approx(2 * 10 / 0.2)


def test_single_rank_is_unchanged():
    import bench
    assert bench.max_over_ranks([3.0, 4.0], 1, torch.device("cpu")) == [3.0, 4.0]
    assert bench.job_rate(1, 5, 500.0) == pytest.approx(10.0)
