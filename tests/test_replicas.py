"""Replica placement and the cross-rank reduction, on CPU with gloo (world size 2)."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from sparqc_gb300 import circuits, replicas


def _batch(n=64):
    return [(nq, g) for nq, _, g in circuits.batch_circuits(n, seed=3, drange=(20, 120))]


def test_shards_partition_the_circuits():
    cs = _batch()
    for world in (1, 2, 3, 8):
        shards = [replicas.shard(cs, r, world) for r in range(world)]
        flat = sorted(i for s in shards for i in s)
        assert flat == list(range(len(cs)))
        assert replicas.imbalance(cs, world) < 1.35
    with pytest.raises(ValueError):
        replicas.shard(cs, 2, 2)


def test_cost_bound_matches_generator():
    # circuits of the batching configuration keep every bit >= k fixed: at most 2^k keys
    for nq, k, g in circuits.batch_circuits(16, seed=5, drange=(20, 80)):
        _, work = replicas.circuit_cost(nq, g)
        assert work <= (2 ** k) * len(g)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    cs = _batch(32)
    mine = replicas.shard(cs, rank, world)
    work = sum(replicas.circuit_cost(*cs[i])[1] for i in mine)
    t, w = replicas.reduce_step(0.5 + rank, work)
    q.put((rank, mine, t, w))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_reduction_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    out.sort()
    cs = _batch(32)
    total = sum(replicas.circuit_cost(*c)[1] for c in cs)
    assert sorted(out[0][1] + out[1][1]) == list(range(32))
    for _, _, t, w in out:
        assert t == 1.5 and w == total
