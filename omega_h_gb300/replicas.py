"""Replica runs over torch.distributed.

The adapt pass does not shard (one mesh's pass needs ghosting and exchanges
after every round), so N GPUs run N independent replicas: each rank adapts
its own meshes with no collective on the data path.  The only exchange is
for timing: a throughput is the units of all ranks over the slowest rank's
time.  With the NCCL backend the reduction runs on the rank's GPU; with gloo
on the CPU.
"""
import torch
import torch.distributed as dist


def world_size():
    return dist.get_world_size() if dist.is_available() and dist.is_initialized() else 1


def max_over_ranks(x, device="cpu"):
    """The largest x over all ranks (x itself on one rank)."""
    if world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(units_per_rank, seconds, device="cpu"):
    """(units of all ranks / the slowest rank's seconds, those seconds)."""
    s = max_over_ranks(seconds, device)
    return world_size() * units_per_rank / s, s
