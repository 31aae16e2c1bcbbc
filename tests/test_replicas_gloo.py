"""The N > 1 path of bench.py on CPU: two gloo ranks (replicas only, no data-path collective).

Every rank runs the whole workload; the step time is the slowest rank's (MAX all-reduce) and the
throughput counts one right-hand side per rank and step.  The reference arm under torchrun runs
on rank 0 only; the other ranks exit 0 without work.
"""
import importlib.util
import os
import socket
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _bench():
    spec = importlib.util.spec_from_file_location("bench_mod", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, q):
    import torch
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench = _bench()
        mine = 0.5 + rank  # rank 1 is the slower replica
        t = bench.max_over_ranks(mine, dist, torch.device("cpu"))
        q.put((rank, t, bench.replica_throughput(world, t)))
    finally:
        dist.destroy_process_group()


def test_step_time_is_the_slowest_replica():
    import torch.multiprocessing as mp

    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(world))
    for rank, t, value in got:
        assert t == pytest.approx(1.5)          # max over the ranks
        assert value == pytest.approx(2 / 1.5)  # two replicas per slowest step


def test_single_rank_needs_no_collective():
    bench = _bench()
    assert bench.max_over_ranks(0.25, None, None) == 0.25
    assert bench.replica_throughput(1, 0.25) == pytest.approx(4.0)


def test_reference_arm_other_ranks_exit_without_work(monkeypatch):
    import argparse

    bench = _bench()
    monkeypatch.setenv("RANK", "1")
    ns = argparse.Namespace(impl="reference", gpus=2, steps=1, warmup=0, workload=bench.WORKLOAD)
    assert bench.reference_arm(ns) == 0  # returns at once: no oracle, no output line
