"""Walker sharding across processes (one GPU each).

Walkers are independent and every random number is keyed by the walker's global index, so a run
splits into contiguous walker ranges with no exchange during the walk; the only collective is the
final sum of the FP64 ensemble partials (Re/Im/second moment per echo and measurement).
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
