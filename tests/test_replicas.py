"""Replica host logic over torch.distributed with gloo, world size 2, on CPU.

A multi-GPU run of this path is N independent replicas: the timings are the only data that
cross ranks (barrier, max over ranks), and a batch of independent systems is sharded so that
every system is solved by exactly one rank.
"""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def worker(rank, ws, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(ws), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    from juesgpu import replicas
    from juesgpu.synthetic import batch_specs
    r = replicas.setup("gloo")
    try:
        r.barrier()
        m = r.max(float(rank) * 10.0 + 1.5)
        specs = batch_specs(37)
        mine = r.shard(specs)
        out.put((rank, r.world_size, m, [s[3] for s in mine]))
        r.barrier()
    finally:
        r.close()


def test_replicas_gloo_world2():
    ws, port = 2, free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=worker, args=(k, ws, port, q)) for k in range(ws)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(ws))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [ws, ws]
    assert all(r[2] == 11.5 for r in res)                 # max over ranks reaches every rank
    from juesgpu.synthetic import batch_specs
    every = [s[3] for s in batch_specs(37)]
    shares = [r[3] for r in res]
    assert sorted(shares[0] + shares[1]) == sorted(every)   # a partition: each system once
    assert abs(len(shares[0]) - len(shares[1])) <= 1


def test_single_process_is_a_replica_of_one():
    from juesgpu import replicas
    env = {k: os.environ.pop(k) for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK") if k in os.environ}
    try:
        r = replicas.setup()
        assert (r.world_size, r.rank, r.dist) == (1, 0, None)
        assert r.max(3.0) == 3.0 and r.shard([1, 2, 3]) == [1, 2, 3]
        r.barrier()
    finally:
        os.environ.update(env)
