"""The N > 1 path of bench.py on CPU: two gloo ranks time different steps; the job's step time
is the slowest rank's and the job's throughput counts every rank's replica."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = bench.max_over_ranks(10.0 + 5.0 * rank, world, torch.device("cpu"))
    out[rank] = (ms, bench.replica_throughput(1024, world, ms))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank_and_the_summed_work():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    port = _free_port()
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
        assert all(p.exitcode == 0 for p in procs)
        res = dict(out)
    for r in range(2):
        ms, value = res[r]
        assert ms == 15.0                          # max over ranks
        assert value == pytest.approx(2 * 1024 / 0.015)


def test_single_rank_is_unchanged():
    import bench
    assert bench.max_over_ranks(12.5, 1) == 12.5
    assert bench.replica_throughput(256, 1, 10.0) == pytest.approx(25600.0)
