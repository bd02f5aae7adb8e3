"""Multi-GPU replicas: independent units (right-hand-side blocks, whole
graphs) are partitioned across ranks with no data-path collective; only the
timing (max over ranks) and result counts are reduced.  A single graph's solve
is never sharded (it would need a halo exchange per SpMV and an allreduce per
dot product).  The reference scales one graph over an MPI process grid
(redistribute.hpp, SpParMat 2-D layout); that path is out of scope here.
"""
import os

import numpy as np


def dist_env():
    """(world_size, rank, local_rank) from the torchrun environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def block_range(total, world, rank):
    """Contiguous share [lo, hi) of `total` equal units for `rank`."""
    base, extra = divmod(total, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def lpt_partition(weights, world):
    """Longest-processing-time-first assignment of weighted units (graphs by
    nnz) to `world` ranks; returns one list of unit indices per rank, each
    list in ascending unit order."""
    order = np.argsort(-np.asarray(weights, dtype=np.float64), kind="stable")
    load = np.zeros(world)
    parts = [[] for _ in range(world)]
    for u in order:
        r = int(np.argmin(load))
        parts[r].append(int(u))
        load[r] += weights[u]
    return [sorted(p) for p in parts]


def reduce_max(values, device=None):
    """Element-wise max over ranks (identity without an initialised group)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor(values, dtype=torch.float64, device=device)
    if dist.is_available() and dist.is_initialized():
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.cpu().tolist()


def reduce_sum(values, device=None):
    import torch
    import torch.distributed as dist
    t = torch.tensor(values, dtype=torch.float64, device=device)
    if dist.is_available() and dist.is_initialized():
        dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return t.cpu().tolist()
