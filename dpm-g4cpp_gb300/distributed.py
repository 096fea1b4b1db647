"""History sharding across processes (one GPU each).

Histories are independent, so a job shards by history range: rank r of W runs
histories [N r / W, N (r+1) / W) of the job (history h always uses random
stream h, so the union of the shards is exactly the unsharded job). The one
exchange is the final sum of the dose and dose^2 tallies.
"""
import numpy as np

from . import Job


def shard(n, rank, world):
    """(first, count) of rank's share of n histories."""
    first = n * rank // world
    return first, n * (rank + 1) // world - first


def shard_job(job, rank, world):
    first, count = shard(job.histories, rank, world)
    return Job(job.phantom, job.source, count, job.seed, job.first_history + first)


def allreduce_sum(arr, device=None):
    """Sums a numpy tally over all ranks of the default process group."""
    import torch
    import torch.distributed as dist
    t = torch.from_numpy(np.ascontiguousarray(arr, dtype=np.float64))
    if device is not None:
        t = t.to(device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return t.cpu().numpy()
