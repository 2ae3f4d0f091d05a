"""The N > 1 path of bench.py on CPU: replicas whose throughput is N * units / the slowest rank's time, with the
max taken over a two-rank gloo process group, and the reference arm running on rank 0 only."""

import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r took 10 (r + 1) ms per step on 1000 units; the slowest rank sets the whole job's time
        ms, value = bench.replica_throughput(10.0 * (rank + 1), 1000.0, world, torch.device("cpu"))
        s, e2e = bench.replica_throughput(0.5 + rank, 1000.0, world, torch.device("cpu"), per="s")
        out[rank] = (ms, value, s, e2e)
    finally:
        dist.destroy_process_group()


def test_replica_throughput_takes_the_slowest_rank():
    world = 2
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
        res = dict(out)
    assert sorted(res) == [0, 1]
    for ms, value, s, e2e in res.values():
        assert ms == pytest.approx(20.0)
        assert value == pytest.approx(world * 1000.0 / 0.020)
        assert s == pytest.approx(1.5)
        assert e2e == pytest.approx(world * 1000.0 / 1.5)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench

    ms, value = bench.replica_throughput(25.0, 500.0, 1, None)
    assert ms == 25.0 and value == pytest.approx(500.0 / 0.025)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench

    monkeypatch.setenv("RANK", "1")
    args = bench_args(bench)
    assert bench.run_reference(args) == 0
    assert capsys.readouterr().out == ""  # no work and no JSON line off rank 0


def bench_args(bench):
    import argparse

    return argparse.Namespace(config="plain_small", steps=1, warmup=0, gpus=2, impl="reference")
