"""The multi-GPU path of the bench is independent replicas (one simulation
per rank, no data-path collective): the whole-job time is the slowest
rank's, the value is the units of all ranks over it, and only rank 0 runs
the CPU reference arm.  Checked here with two gloo ranks on the host."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

import bench


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t = bench.max_over_ranks(1.0 + rank, dist)      # rank r took 1 + r seconds
        out[rank] = (t, bench.replicas_value(100.0, world, t), bench.dist_setup())
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_replicas_slowest_rank_sets_the_time():
    world = 2
    port = _free_port()
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    for r in range(world):
        t, value, (w, rank, local) = res[r]
        assert t == 2.0                                 # the slowest rank's time on every rank
        assert value == pytest.approx(world * 100.0 / 2.0)
        assert (w, rank, local) == (world, r, r)


def test_single_process_needs_no_group():
    assert bench.max_over_ranks(3.5, None) == 3.5
    assert bench.replicas_value(10.0, 1, 2.0) == 5.0


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("LOCAL_RANK", "1")
    called = []
    monkeypatch.setattr(bench, "cpu_baseline", lambda *a, **k: called.append(1))

    class A:
        procs, warmup, steps, gpus = 1, 1, 1, 2
    bench.run_reference(A())
    assert not called and capsys.readouterr().out == ""
