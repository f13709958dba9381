"""The N > 1 path of bench.py on CPU: independent replicas (one per rank,
gloo here, NCCL on GPUs) whose timings are combined by the slowest rank;
no collective on the data path."""

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
        ms = 10.0 + 5.0 * rank            # rank 1 is the slow replica
        slowest = bench.max_over_ranks(ms, world, "cpu")
        rate = bench.whole_job_rate(1000, world, slowest * 1e-3)
        dist.barrier()
        out[rank] = (slowest, rate)
    finally:
        dist.destroy_process_group()


def test_replicas_take_the_slowest_rank():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        procs = [ctx.Process(target=_rank, args=(r, world, port, out))
                 for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    for r in range(world):
        slowest, rate = res[r]
        assert slowest == 15.0
        assert rate == pytest.approx(1000 * 2 / 0.015)


def test_single_rank_is_local():
    import bench
    assert bench.max_over_ranks(3.5, 1, "cpu") == 3.5
    assert bench.whole_job_rate(10, 1, 2.0) == 5.0
