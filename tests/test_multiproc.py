"""The benchmark's multi-rank host logic (replicas only) on CPU: two gloo
ranks agree on the max-over-ranks time, and the reference arm does its work
on rank 0 only."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    t = bench.max_over_ranks(10.0 + rank * 5.0, world)
    bench.barrier(world)
    r, w, lr = bench.dist_info()
    q.put((rank, t, r, w, lr))
    dist.destroy_process_group()


def test_max_over_ranks_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    assert [g[1] for g in got] == [15.0, 15.0]
    assert [(g[2], g[3], g[4]) for g in got] == [(0, 2, 0), (1, 2, 1)]


def test_reference_arm_nonzero_rank_does_no_work(monkeypatch, capsys):
    import sys

    import bench

    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setattr(sys, "argv", ["bench.py", "--impl", "reference", "--n-points", "1000"])
    bench.main()
    assert capsys.readouterr().out == ""
