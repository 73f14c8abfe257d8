"""Multi-GPU use of the solver: independent replicas.

The reference advances a batched NeuralODE state with ONE step size and ONE
error norm over all trajectories (src/neural_de.jl:52), so splitting a batch
across GPUs would change the solution. Multi-GPU runs are therefore replicas:
each rank solves its own batch (its own controller), and data-parallel
training averages the parameter gradients on the host side of the step --
one collective per step on a P-float vector, none on the solver's data path.
Multiple-shooting segments are independent solves and could be sharded
without changing results; the same gradient average applies.

These helpers only use torch.distributed, so they run with the `gloo`
backend on CPU as well as with `nccl`.
"""
import numpy as np


def rank_world():
    import os
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1"))


def replica_seed(base_seed, rank):
    """Seed of rank `rank`'s independent batch."""
    return int(base_seed) * 1000003 + int(rank)


def shard_segments(nseg, rank, world):
    """Contiguous block of independent segments (multiple shooting) for a rank."""
    per = (nseg + world - 1) // world
    lo = min(nseg, rank * per)
    return range(lo, min(nseg, lo + per))


def average_gradients(grad, group=None):
    """Mean of a parameter-gradient vector over the replicas (in place for
    torch tensors; returns a new array for numpy input)."""
    import torch
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized():
        return grad
    world = dist.get_world_size(group)
    t = grad if isinstance(grad, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(grad))
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    t /= world
    return t if isinstance(grad, torch.Tensor) else t.numpy()


def sum_over_ranks(x, group=None):
    """Sum of a vector (or scalar) over the ranks: the multiple-shooting loss
    and its gradient are sums over trajectories, so sharding trajectories
    across ranks needs a sum, not a mean. Returns a new numpy array / float."""
    import torch
    import torch.distributed as dist
    scalar = np.ndim(x) == 0
    a = np.atleast_1d(np.asarray(x, dtype=np.float64)).copy()
    if not dist.is_available() or not dist.is_initialized():
        return float(a[0]) if scalar else a
    t = torch.from_numpy(a)
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return float(t[0]) if scalar else t.numpy()


def max_over_ranks(value, group=None):
    """Largest value over the replicas (step time of a synchronised step)."""
    import torch
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized():
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())
