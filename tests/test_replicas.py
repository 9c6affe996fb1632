"""The multi-rank (replica) bookkeeping on CPU: two gloo ranks, no GPU.

Each rank runs an independent replica; the job's step time is the slowest
rank's and its throughput is the units of all ranks over that time.  A batch
of molecules is split round-robin with no unit lost or duplicated.
"""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from rest_tensors_gb300 import replicas  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        local_ms = 10.0 + 5.0 * rank           # rank 1 is the slow one
        ms = replicas.max_over_ranks(local_ms)
        mine = replicas.shard(list(range(64)), rank, world)
        got = [None] * world
        dist.all_gather_object(got, mine)
        q.put((rank, ms, got))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time_and_split_molecules():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, ms, parts in res:
        assert ms == 15.0
        flat = sorted(x for part in parts for x in part)
        assert flat == list(range(64))
        assert set(parts[0]).isdisjoint(parts[1])


def test_single_process_helpers():
    assert replicas.max_over_ranks(3.5) == 3.5
    assert replicas.shard([1, 2, 3, 4, 5], 1, 2) == [2, 4]
    assert replicas.job_throughput([3e11, 3e11], 0.01) == pytest.approx(6e13)
    with pytest.raises(ValueError):
        replicas.shard([1], 2, 2)
