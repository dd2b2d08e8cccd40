"""Replica plumbing on CPU ranks (gloo, world size 2): the job partition is
disjoint, complete and balanced without communication, and the cross-rank
reductions give the slowest rank's time and the whole job's pixel count."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, costs, q):
    import torch.distributed as dist
    from tucuda_gb300 import replicas
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mine = replicas.shard(costs, rank, world)
        pixels = sum(costs[i] for i in mine)
        step_ms = 1.0 + rank  # rank 1 is the slow one
        replicas.barrier()
        q.put((rank, mine, replicas.max_over_ranks(step_ms), replicas.sum_over_ranks(pixels),
               replicas.rank_world()))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks():
    import torch.multiprocessing as mp
    costs = [1920 * 1080, 640 * 480, 4096 * 2160, 320 * 240, 1280 * 720, 3840 * 2160, 800 * 600]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, costs, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, m0, mx0, sm0, rw0), (r1, m1, mx1, sm1, rw1) = res
    assert (r0, r1) == (0, 1) and rw0 == (0, 2) and rw1 == (1, 2)
    assert not set(m0) & set(m1) and sorted(m0 + m1) == list(range(len(costs)))
    loads = [sum(costs[i] for i in m) for m in (m0, m1)]
    assert max(loads) <= sum(costs) - min(loads)  # no rank holds everything
    assert mx0 == mx1 == 2.0
    assert sm0 == sm1 == float(sum(costs))


def test_single_process_defaults():
    from tucuda_gb300 import replicas
    assert replicas.rank_world() == (0, 1)
    assert replicas.max_over_ranks(3.5) == 3.5
    assert replicas.shard([5, 3, 1], 0, 1) == [0, 1, 2]
    with pytest.raises(ValueError):
        replicas.shard([1], 2, 2)
