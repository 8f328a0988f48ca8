"""Host logic of the N > 1 bench path on CPU: replicas over a gloo process
group (world size 2, rendezvous on 127.0.0.1). The step is not sharded:
every rank runs its own copy of the workload, the job's time is the slowest
rank's and its work the sum over ranks; the reference arm runs on rank 0
only."""
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


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, local = bench.dist_env()
        # rank-dependent time and work, as unequal replicas would report
        t_ms = 10.0 + 5.0 * r
        units = 1000 * (r + 1)
        t_max, tot = bench.reduce_over_ranks(t_ms, units, w, "cpu")
        out[r] = (r, w, local, t_max, tot)
    finally:
        dist.destroy_process_group()


def test_reduce_over_ranks_gloo_world2():
    world = 2
    # the manager's server process is started with spawn, as the ranks are
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(world, _free_port(), out), nprocs=world, join=True)
    assert sorted(out.keys()) == [0, 1]
    for r in range(world):
        rr, w, local, t_max, tot = out[r]
        assert (rr, w, local) == (r, world, r)
        assert t_max == 15.0          # the slowest rank
        assert tot == 3000.0          # work of both replicas


def test_reduce_over_ranks_single_process():
    assert bench.reduce_over_ranks(12.5, 77, 1, "cpu") == (12.5, 77)


def test_reference_arm_runs_on_rank0_only(monkeypatch, capsys):
    """A rank other than 0 returns before any work and prints nothing."""
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("LOCAL_RANK", "1")

    class Args:
        steps, warmup, gpus = 1, 0, 2

    bench.run_reference(Args(), bench.WORKLOADS["turb3d"])
    assert capsys.readouterr().out == ""


def test_workload_sort_interval_defaults():
    """Sort cadence is per workload unless given on the command line."""
    assert bench.WORKLOADS["turb3d"]["sort_interval"] == 8
    assert bench.WORKLOADS["pair2d"]["sort_interval"] == 16
    assert bench.WORKLOADS["wald2d"]["sort_interval"] == 0
