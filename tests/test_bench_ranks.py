"""bench.py with N > 1 ranks (replicas): two gloo ranks on the CPU.

Each rank times its own replica; the job's time is the slowest rank's
(max over ranks) and the job's value counts every rank's particle-steps
over that time.  The GPU runs use NCCL with the same calls.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        local_ms = [10.0, 14.5][rank]
        el_ms = bench.max_over_ranks(local_ms, dist, "cpu")
        value = bench.job_value(1000 * 20, world, el_ms * 1e-3)
        dist.barrier()
        out.put((rank, el_ms, value))
    finally:
        dist.destroy_process_group()


def test_two_ranks_take_the_slowest_time_and_add_the_units():
    import torch.multiprocessing as mp
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(out.get(timeout=10) for _ in range(2))
    for rank, el_ms, value in got:
        assert el_ms == 14.5                          # the slower rank's time on both
        assert value == pytest.approx(2 * 1000 * 20 / 14.5e-3)


def test_single_process_passes_its_own_time():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.25, None, "cpu") == 3.25
    assert bench.job_value(500, 1, 0.5) == 1000.0
