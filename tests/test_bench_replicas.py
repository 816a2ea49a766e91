"""The multi-GPU path of bench.py is replicas only (every rank advances its own pulse, no
data-path collective): the job's time is the slowest rank's (an all-reduce MAX over the process
group) and its value all ranks' field-point z-steps over that time; the reference arm runs on
rank 0 alone.  Checked here with two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        ms, value = bench.whole_job(10.0 * (rank + 1), 1000, world)   # rank 1 is the slower
        out[rank] = (ms, value)
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_whole_job_is_the_slowest_rank_and_all_units():
    world = 2
    out = mp.Manager().dict()
    mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
    for r in range(world):
        ms, value = out[r]
        assert ms == 20.0                       # the max over ranks, on every rank
        assert value == pytest.approx(1000 * world / 0.020)


def test_single_process_needs_no_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.whole_job(5.0, 1000, 1) == (5.0, pytest.approx(1000 / 0.005))


def test_reference_arm_runs_on_rank_0_only(capsys):
    sys.path.insert(0, ROOT)
    import bench

    class A:   # the arguments reference_arm reads before any work
        workload = "c2"

    bench.reference_arm(A(), rank=1, world=2)   # rank 1 returns at once, printing nothing
    assert capsys.readouterr().out == ""
