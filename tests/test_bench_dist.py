"""bench.py's multi-rank plumbing on CPU (gloo, world size 2): the replicas'
clocks are combined by one max all_reduce, the reference arm runs on rank 0
only, and the rank / world come from the torchrun environment."""
from __future__ import annotations

import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, port, out):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2",
                      LOCAL_RANK=str(rank))
    import bench

    world, r, local = bench.dist_setup()
    dist.init_process_group("gloo", rank=r, world_size=world)
    # rank 0 measured (1.0 s device, 5.0 s end to end), rank 1 (2.0 s, 4.0 s)
    vals = bench.replica_max([1.0 + rank, 5.0 - rank], world)
    dist.destroy_process_group()
    out.put((rank, world, local, vals))


def test_replica_clocks_take_the_max_over_two_gloo_ranks():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[:3] for g in got] == [(0, 2, 0), (1, 2, 1)]
    for _, _, _, vals in got:
        assert vals == [2.0, 5.0]


def test_single_rank_needs_no_process_group():
    import bench

    assert bench.replica_max([3.0, 7.0], 1) == [3.0, 7.0]


def test_reference_arm_is_rank_zero_only(capsys):
    import bench

    # a non-zero rank returns before any work or output (its arguments are
    # never read)
    bench.run_reference(None, 2, 1)
    assert capsys.readouterr().out == ""
