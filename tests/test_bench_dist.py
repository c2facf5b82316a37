"""The multi-rank path of bench.py on the CPU: two gloo ranks (as torchrun
launches them) agree on the slowest rank's time, the whole-job value
scales with the number of ranks (weak scaling), and the reference arm runs
on rank 0 alone."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        dist.barrier()
        ms = bench.max_over_ranks(10.0 + 5.0 * rank, dist, "cpu")
        # the reference arm: a rank other than 0 returns without work or output
        if rank != 0:
            class A:  # the parsed arguments the reference arm reads
                cpu_log2n, warmup, steps = 30, 0, 1
            bench.run_reference(A(), rank, world)
        q.put((rank, ms))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=5) for _ in range(2))
    assert got == [(0, 15.0), (1, 15.0)]


def test_aggregate_is_weak_scaling():
    import bench
    one = bench.aggregate_gbs(1, 2e9, 4, 8.0)
    assert one == pytest.approx(1000.0)
    assert bench.aggregate_gbs(4, 2e9, 4, 8.0) == pytest.approx(4 * one)
    assert bench.max_over_ranks(3.5, None, "cpu") == 3.5
