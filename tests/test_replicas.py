"""Replica aggregation of bench.py --gpus N, as two gloo ranks on the CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from polymps_gb300 import replicas
    units, secs = replicas.aggregate(1000 * (rank + 1), 0.5 * (rank + 1), world)
    replicas.barrier(world)
    q.put((rank, units, secs))
    dist.destroy_process_group()


def test_replica_aggregation_two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = [q.get(timeout=120) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, units, secs in got:
        assert units == 3000.0      # particle-steps of both replicas
        assert secs == 1.0          # the slower replica's time


def test_replica_aggregation_single_rank():
    from polymps_gb300 import replicas
    assert replicas.aggregate(123, 0.25, 1) == (123.0, 0.25)
