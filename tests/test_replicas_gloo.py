"""The N > 1 bench path without GPUs: two gloo ranks on the CPU run the replica timing
reduction of bench.py (barrier, max over ranks) and the whole-job value, and the
reference arm does its work on rank 0 only."""

import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = bench.replica_max_ms(10.0 + 5.0 * rank, torch.device("cpu"), world)
    value = bench.replica_value(1000, 20, world, ms)
    out.put((rank, ms, value))
    dist.destroy_process_group()


def test_two_rank_replica_timing_takes_the_slowest_rank():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [15.0, 15.0]
    assert all(r[2] == pytest.approx(1000 * 20 * 2 / 0.015 / 1e6) for r in res)


def test_reference_arm_is_rank_zero_only(capsys):
    import sys
    sys.path.insert(0, ROOT)
    import bench

    class A:
        steps, warmup, gpus = 1, 1, 2
    bench.run_reference(A, rank=1, world=2)
    assert capsys.readouterr().out == ""
