"""The multi-rank side of bench.py on CPU (gloo, world size 2): max over ranks, whole-job value,
and the reference arm's non-zero ranks exiting without work."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        ms = bench.reduce_max(10.0 + 5.0 * rank, world)  # rank 1 is the slower one
        out[rank] = (ms, bench.replica_value(1000, ms, world))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_reduce_max_and_value_two_ranks():
    world = 2
    out = mp.Manager().dict()
    mp.spawn(_worker, args=(world, _free_port(), out), nprocs=world, join=True)
    for rank in range(world):
        ms, value = out[rank]
        assert ms == 15.0
        assert value == pytest.approx(2 * 1000 / 0.015)


def test_reference_arm_other_ranks_do_nothing(capsys):
    sys.path.insert(0, ROOT)
    import bench

    class Args:
        warmup, steps, gpus = 1, 1, 2
    assert bench.run_reference(Args(), bench.WORKLOADS["small"], rank=1, world=2) is None
    assert capsys.readouterr().out == ""


def test_single_rank_reduce_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.reduce_max(3.5, 1) == 3.5
    assert bench.replica_value(100, 10.0, 1) == pytest.approx(1e4)
