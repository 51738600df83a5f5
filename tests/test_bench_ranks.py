"""The multi-rank host logic of bench.py on CPU: replicas on a gloo process
group of two ranks report the whole job's throughput over the slowest
rank's time (the same function the GPU runs use under torchrun/NCCL)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        bench.barrier(world)
        # rank r took (r + 1) * 10 ms for 1000 children
        value, total_ms = bench.job_value(1000, (rank + 1) * 10.0, world)
        out[rank] = (value, total_ms)
        bench.barrier(world)
    finally:
        dist.destroy_process_group()


def test_job_value_is_max_over_two_gloo_ranks():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    for r in range(world):
        value, total_ms = res[r]
        assert total_ms == 20.0                       # the slowest rank
        assert value == pytest.approx(2 * 1000 / 0.020)  # all ranks' children / that time


def test_job_value_single_rank():
    import bench
    value, total_ms = bench.job_value(500, 5.0, 1)
    assert (value, total_ms) == (pytest.approx(1e5), 5.0)
