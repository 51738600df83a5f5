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


def _reference_arm(rank, world):
    import json
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    r = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--impl", "reference", "--gpus", str(world),
                        "--steps", "1", "--warmup", "0"], capture_output=True, text=True, timeout=600, env=env,
                       cwd=root)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    return [json.loads(ln) for ln in lines]


def test_reference_arm_prints_the_contract_line_on_rank_0_only():
    """bench.py --impl reference times the CPU implementation of the rule
    step on the host cores: rank 0 prints one JSON line with the bench's
    metric, a cpu_baseline and an e2e of zero copies; other ranks print
    nothing and exit 0."""
    (line,) = _reference_arm(0, 2)
    assert line["impl"] == "reference"
    assert line["metric"] == "child objects/s per simulate() step" and line["unit"] == "children/s"
    assert line["value"] > 0 and line["higher_is_better"] is True
    assert (line["n_gpus"], line["steps"], line["warmup"]) == (2, 1, 0)
    cb = line["cpu_baseline"]
    assert cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": "children/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert "workload" in line["config"]
    assert _reference_arm(1, 2) == []
