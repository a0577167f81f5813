"""The replica path of bench.py (one process per GPU, no collective on the data path): the
whole-job throughput counts every rank's paths over the slowest rank's time. Two gloo
ranks on the CPU stand in for two GPUs."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms_local = [100.0, 250.0][rank]  # rank 1 is slower
    value, t_max = bench.job_throughput(1000, 5, world, ms_local, device="cpu")
    q.put((rank, value, t_max))
    dist.barrier()
    dist.destroy_process_group()


def test_job_throughput_over_two_ranks():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(world))
    for rank, value, t_max in res:
        assert t_max == pytest.approx(250.0)
        assert value == pytest.approx(1000 * 5 * 2 / 0.25)


def test_single_rank_is_local_time():
    import bench
    assert bench.job_throughput(10, 2, 1, 40.0) == (pytest.approx(500.0), 40.0)
