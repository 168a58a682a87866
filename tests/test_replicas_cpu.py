"""The N>1 path of bench.py: every rank advances its own replica and the timed
region is the maximum over ranks (replicas only: the step does not shard).
Exercised with two gloo ranks on the CPU."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    t = bench.reduce_max(0.5 + rank, world, device="cpu")
    world_, rank_, local_ = bench._dist()
    q.put((rank, t, world_, rank_))
    dist.destroy_process_group()


def test_two_rank_max_timing():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
    assert [o[1] for o in out] == [1.5, 1.5]
    assert [(o[2], o[3]) for o in out] == [(2, 0), (2, 1)]
