"""One Monte Carlo run sharded over processes (one GPU each): contiguous path ranges, one exact
sum-reduce of the integer accumulators.

The paths of a run are independent and each process positions its random numbers at its own
first path (mrg32k3a skip-ahead, Sobol index offset), so the shards together simulate exactly
the paths of one unsharded run.  Every sum of the run is an exact integer (fixed point in
pairs of int64 words), so adding the shards' words is exact and the finished results are bit-
identical to one call over all the paths, whatever the number of shards and the order of the
reduction.  This is the sharding of mcParallelSimul's path loop (mcBase.h:331-400) across
devices, with one collective at the end instead of the per-thread result vectors.
"""
import numpy as np

from .api import results_from_raw

ALIGN = 64  # shards start on multiples of 64 paths: antithetic pairs and Sobol warp batches stay whole


def shard_range(n_path, rank, world):
    """(firstPath, numPath) of shard `rank` of `world` over a run of n_path paths: contiguous
    ranges in rank order, each start a multiple of 64, sizes as even as that allows (a shard
    may be empty when n_path is small)."""
    if world < 1 or not 0 <= rank < world or n_path < 0:
        raise ValueError("bad shard")
    blocks = -(-n_path // ALIGN)
    b0, b1 = blocks * rank // world, blocks * (rank + 1) // world
    first = min(n_path, b0 * ALIGN)
    last = min(n_path, b1 * ALIGN)
    return first, last - first


def combine(acc, group=None):
    """Word-wise int64 sum of the shards' accumulators over the process group (all ranks get
    the total).  Integer addition: exact and independent of the reduction order."""
    import torch
    import torch.distributed as dist
    t = torch.from_numpy(np.ascontiguousarray(acc, dtype=np.int64))
    if dist.get_backend(group) == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t.cpu().numpy()


def run_shard(eng, modelId, productId, num, rank, world, risk=True, weights=None, group=None):
    """This process's shard of a run of num.numPath paths, the exact reduction, and the
    finished results of the whole run: (values, stderrs, aggregate, risks)."""
    from dataclasses import replace
    npay, npar, _ = eng.shapes(modelId, productId)
    first, count = shard_range(num.numPath, rank, world)
    nwords = 2 * ((npar if risk else 0) + 2 * npay + 2)
    if count > 0:
        eng.enqueue_shard(modelId, productId, replace(num, numPath=count), first, risk=risk, weights=weights)
        acc = eng.fetch_raw()
    else:
        acc = np.zeros(nwords, dtype=np.int64)
    total = combine(acc, group) if world > 1 else acc
    return results_from_raw(total, npar if risk else 0, npay, num.numPath)
