"""Walker and instance sharding across processes (one GPU each).

Walkers are independent and every random number is keyed by the walker's global index, so a run
splits into contiguous walker ranges with no exchange during the walk; the only collective is the
final sum of the FP64 ensemble partials (Re/Im/second moment per echo and measurement).  A batch
of instances shards by instance: each rank walks a cost-balanced subset and the signals are
gathered at the end.
"""
import numpy as np


def shard_range(n_walkers, world_size, rank):
    """(walker_offset, count) of ``rank``'s contiguous share of ``n_walkers``."""
    if world_size < 1 or not 0 <= rank < world_size:
        raise ValueError("need 0 <= rank < world_size")
    base, extra = divmod(int(n_walkers), int(world_size))
    offset = rank * base + min(rank, extra)
    return offset, base + (1 if rank < extra else 0)


def allreduce_sums(sums, group=None):
    """Sum the (n_echo, M, 3) FP64 partial sums of every rank (torch.distributed, any backend)."""
    import torch
    import torch.distributed as dist
    t = torch.as_tensor(np.asarray(sums, dtype=np.float64))
    dev = torch.device("cuda", torch.cuda.current_device()) \
        if dist.get_backend(group) == "nccl" else torch.device("cpu")
    t = t.to(dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t.cpu().numpy()


def shard_instances(costs, world_size, rank):
    """Indices of the instances ``rank`` walks: greedy longest-processing-time assignment of the
    per-instance costs (walker-steps) to ``world_size`` ranks, so every rank gets about the same
    work; every instance goes to exactly one rank, the same on every rank."""
    if world_size < 1 or not 0 <= rank < world_size:
        raise ValueError("need 0 <= rank < world_size")
    order = sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i))
    load = [0.0] * world_size
    mine = []
    for i in order:
        r = min(range(world_size), key=lambda k: (load[k], k))
        load[r] += float(costs[i])
        if r == rank:
            mine.append(i)
    return sorted(mine)


def gather_signals(local, indices, n_total, group=None):
    """Assemble every rank's {instance index: signal array} into one list in instance order
    (torch.distributed all_gather_object, any backend)."""
    import torch.distributed as dist
    world = dist.get_world_size(group)
    parts = [None] * world
    dist.all_gather_object(parts, [(int(i), np.asarray(s)) for i, s in zip(indices, local)],
                           group=group)
    out = [None] * n_total
    for part in parts:
        for i, sig in part:
            out[i] = sig
    return out
