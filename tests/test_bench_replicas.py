"""bench.py on CPU: the multi-rank side (gloo, world size 2: max over ranks, whole-job value, the
reference arm's non-zero ranks exiting without work) and the reference arm's JSON line."""
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


def test_reference_arm_line_keeps_the_contract():
    """`bench.py --impl reference` (the CPU arm: the oracle's full plain-method fit of the pair,
    nothing extrapolated) prints one JSON line with the keys the GPU arm's line carries."""
    import json
    import subprocess
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", "small",
                          "--steps", "1", "--warmup", "0"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    rec = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
                "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert key in rec, key
    assert rec["impl"] == "reference" and rec["higher_is_better"] is True and rec["steps"] == 1
    assert rec["metric"] == rec["unit"] == "query patches/s"
    assert rec["value"] == pytest.approx((512 - 7 + 1) ** 2 / (rec["ms_per_step"] / 1e3), rel=1e-6)
    assert rec["cpu_baseline"]["value"] == rec["value"] and rec["cpu_baseline"]["cores"] >= 1
    assert rec["cpu_baseline"]["kind"] in ("port", "reference")
    assert rec["e2e"] == {"value": rec["value"], "unit": rec["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert "workload" in rec["config"]
