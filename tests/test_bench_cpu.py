"""The benchmark's multi-GPU bookkeeping on CPU.

`bench.py --gpus N` runs one replica of the workload per rank (no data-path
collective): each rank times its own timesteps, the job's time is the
slowest rank's (an all-reduce of the seconds with MAX), and `value` counts
the agent-steps of all replicas.  The reference arm runs on rank 0 only.
The collective is exercised here with two gloo ranks on 127.0.0.1.
"""
import argparse
import os
import socket
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)

import bench  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out_dir):
    import torch.distributed as dist
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    # rank r timed 1.5 + r seconds for its replica
    seconds = bench.slowest_rank_seconds(1.5 + rank, world, device="cpu")
    rate = bench.job_rate(world, 1048576, 100, seconds)
    with open(os.path.join(out_dir, f"rank{rank}.txt"), "w") as f:
        f.write(f"{seconds} {rate}")
    dist.barrier()
    dist.destroy_process_group()


def test_job_time_is_the_slowest_rank_over_gloo(tmp_path):
    import torch.multiprocessing as mp
    world = 2
    mp.start_processes(_rank, args=(world, _free_port(), str(tmp_path)), nprocs=world,
                       start_method="spawn")
    for r in range(world):
        seconds, rate = map(float, (tmp_path / f"rank{r}.txt").read_text().split())
        assert seconds == 2.5
        assert rate == pytest.approx(2 * 1048576 * 100 / 2.5)


def test_single_rank_needs_no_collective():
    assert bench.slowest_rank_seconds(0.8, 1) == 0.8
    assert bench.job_rate(1, 1000, 10, 2.0) == 5000.0


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("LOCAL_RANK", "1")
    args = argparse.Namespace(steps=1, warmup=0, gpus=2, impl="reference", cpu_seconds=1.0)
    assert bench.run_reference(args) == 0
    assert capsys.readouterr().out == ""
