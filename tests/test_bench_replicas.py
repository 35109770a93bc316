"""The multi-GPU path of bench.py is "replicas only": every rank runs one
full solver, the ranks meet at a barrier, and the timed region is the
maximum over ranks; the job value counts every rank's face-updates.  These
checks run that reduction with two gloo ranks on CPU."""
import os
import socket
import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, secs, out):
    import torch
    import torch.distributed as dist

    sys.path.insert(0, str(REPO))
    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        dist.barrier()
        m = bench.max_over_ranks(torch, secs[rank], world, "cpu")
        out[rank] = (m, bench.job_value(1000, 10, world, m))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    manager = ctx.Manager()
    out = manager.dict()
    secs = [0.25, 0.5]
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, secs, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    assert out[0] == out[1] == (0.5, 1000 * 10 * 2 / 0.5)


def test_single_rank_is_identity():
    torch = pytest.importorskip("torch")
    sys.path.insert(0, str(REPO))
    import bench

    assert bench.max_over_ranks(torch, 0.3, 1, "cpu") == 0.3
    assert bench.job_value(163842, 200, 1, 0.02) == 163842 * 200 / 0.02


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    """Under torchrun the reference arm's other ranks exit without work."""
    sys.path.insert(0, str(REPO))
    import argparse

    import bench

    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    args = argparse.Namespace(gpus=2, steps=1, warmup=1, impl="reference")
    assert bench.run_reference(args) is None
    assert capsys.readouterr().out == ""
