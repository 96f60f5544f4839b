"""The N > 1 path of bench.py on CPU: world_size-2 gloo process groups.

bench.py runs independent replicas per rank (the eSRRF path shards by stack /
timepoint with no data exchange); ranks only meet in a barrier and in the
max-over-ranks timing reduction, and in the reference arm only rank 0 works.
"""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

import bench


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        dist.barrier()
        got = bench.max_over_ranks(10.0 * (rank + 1))
        q.put((rank, got))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_with_gloo_world_size_2():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == {0: 20.0, 1: 20.0}


def test_max_over_ranks_without_process_group_is_identity():
    assert bench.max_over_ranks(3.5) == 3.5


def test_reference_arm_non_zero_rank_exits_without_work(monkeypatch, capsys):
    monkeypatch.setenv("RANK", "1")

    class A:
        gpus, steps, warmup = 2, 1, 0

    assert bench.run_reference_arm(A()) == 0
    assert capsys.readouterr().out == ""
