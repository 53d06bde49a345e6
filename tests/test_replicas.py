"""The multi-GPU path of bench.py is replicas: each rank evaluates its own batch; the timed region ends with the
slowest rank (max over ranks) and the throughput counts the evaluations of all ranks. Checked here with two gloo
ranks on the CPU (no GPU, no collective on the data path)."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, times, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t = bench.max_over_ranks(times[rank], dist)
    out.put((rank, t, bench.throughput(161, 10, world, t)))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_and_throughput_gloo():
    pytest.importorskip("torch")
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    times = [0.25, 0.40]
    procs = [ctx.Process(target=_rank, args=(r, 2, port, times, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, v in res:
        assert t == 0.40
        assert abs(v - 161 * 10 * 2 / 0.40) < 1e-9


def test_single_rank_passthrough():
    import bench
    assert bench.max_over_ranks(0.3, None) == 0.3
    assert bench.throughput(4, 5, 1, 2.0) == 10.0
