"""Replica runs of the per-step path on N GPUs of one node.

The path does not shard (every box of this setup has one GPU), so ``bench.py --gpus N``
runs N independent replicas, one per rank, with no collective on the data path.  The
job's throughput is the particle-steps of all ranks over the slowest rank's device time;
the only collectives are the two scalar reductions below and the barriers around the
timed region.
"""
import torch
import torch.distributed as dist


def aggregate(units, seconds, world, device="cpu"):
    """(sum of units over ranks, max of seconds over ranks); identity for one rank."""
    if world <= 1:
        return float(units), float(seconds)
    u = torch.tensor([float(units)], dtype=torch.float64, device=device)
    s = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    dist.all_reduce(s, op=dist.ReduceOp.MAX)
    return float(u.item()), float(s.item())


def barrier(world):
    if world > 1:
        dist.barrier()
