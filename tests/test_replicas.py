"""The multi-GPU path of bench.py is replicas only: each rank times its own system and the
whole-job value is world x units x steps over the slowest rank's time.  Checked here with two
gloo ranks on the CPU (no GPU), as the NCCL run on N GPUs does it."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    # rank r was slower by r x 10 ms; every rank must report the slowest time
    total_ms, value = bench.replica_throughput(100.0 + 10.0 * rank, 1.0e6, 50, world, "cpu")
    dist.barrier()
    out[rank] = (total_ms, value)
    dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank():
    world = 2
    port = _free_port()
    out = mp.Manager().dict()
    mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
    for r in range(world):
        total_ms, value = out[r]
        assert total_ms == pytest.approx(110.0)
        assert value == pytest.approx(world * 1.0e6 * 50 / 0.110)


def test_single_replica_needs_no_process_group():
    import bench

    total_ms, value = bench.replica_throughput(200.0, 1.0e6, 10, 1)
    assert total_ms == 200.0
    assert value == pytest.approx(1.0e6 * 10 / 0.2)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    """Under torchrun the reference arm (host cores) runs once, on rank 0; other ranks exit
    without work or output."""
    import argparse

    import bench

    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("LOCAL_RANK", "1")
    bench.run_reference(argparse.Namespace(steps=1, warmup=1, gpus=2, impl="reference"))
    assert capsys.readouterr().out == ""
