"""Multi-rank host logic of bench.py on CPU (gloo, world size 2).

The workload does not exchange data between ranks: replicas of C0-C2 and
shards of the C3 ensemble run independently, and the only collective is the
MAX over ranks of the timed durations. Here two gloo ranks check that
reduction, the specimen sharding (every specimen exactly once, in order) and
that the reference arm and the adjoint run on rank 0 only.
"""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

import bench  # noqa: E402


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    # each rank's own (ms, e2e seconds); the slowest rank decides
    mine = [10.0 + rank, 3.0 - rank]
    out[rank] = bench.max_over_ranks(mine, world, "cpu")
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_with_two_gloo_ranks():
    world, port = 2, free_port()
    out = mp.get_context("spawn").Manager().dict()
    mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
    assert out[0] == out[1] == [11.0, 3.0]


def test_max_over_ranks_single_rank_is_identity():
    assert bench.max_over_ranks([1.5, 2.5], 1, "cpu") == [1.5, 2.5]


@pytest.mark.parametrize("n,world", [(1024, 2), (1024, 3), (7, 4), (3, 8)])
def test_shards_cover_every_specimen_once(n, world):
    got = []
    for r in range(world):
        lo, hi = bench.shard(n, r, world)
        assert 0 <= lo <= hi <= n
        got.extend(range(lo, hi))
    assert got == list(range(n))


def test_reference_arm_and_adjoint_run_on_rank_zero_only(monkeypatch, capsys):
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("LOCAL_RANK", "1")

    class Args:
        config = 0
        scale = None
        steps = 1
        warmup = 1
        adj_steps = 10
        every = 0

    assert bench.run_reference(Args()) is None
    assert bench.run_adjoint(Args()) is None
    assert capsys.readouterr().out == ""
