"""The multi-rank logic of bench.py on the CPU: two gloo ranks agree on the slowest rank's
time and on the whole job's throughput (every rank sorts its own replica of the workload),
and under a multi-rank launch only rank 0 of the reference arm prints."""

import os
import socket
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out_dir):
    import torch
    import torch.distributed as dist

    sys.path.insert(0, str(ROOT))
    import bench

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        ms, value = bench.job_throughput(torch, [10.0, 14.0][rank], 1000, world, "cpu")
    finally:
        dist.destroy_process_group()
    Path(out_dir, f"rank{rank}.txt").write_text(f"{ms} {value}")


def test_two_gloo_ranks_take_the_slowest_time(tmp_path):
    import torch.multiprocessing as mp

    port = _free_port()
    mp.start_processes(_rank, args=(2, port, str(tmp_path)), nprocs=2, join=True, start_method="spawn")
    for rank in range(2):
        ms, value = (float(x) for x in Path(tmp_path, f"rank{rank}.txt").read_text().split())
        assert ms == 14.0
        assert value == pytest.approx(2 * 1000 / 0.014)


def test_reference_arm_prints_on_rank_0_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--gpus", "2", "--steps", "1",
                        "--warmup", "1"], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
