"""Running the engine on several GPUs at once: host-side logic.

The TSDF path shards by independent objects: each rank (one process per GPU)
integrates and meshes its own volumes, and nothing is exchanged on the data
path.  What the ranks share is bookkeeping: which scenes a rank takes when a
fixed set of scenes is split across GPUs (balanced by voxel-updates), a
barrier before a timed region, and the slowest rank's elapsed time and the
total work for a whole-job rate.  The collectives go through
torch.distributed (NCCL between GPUs, gloo on CPU); with one process every
function here is the identity.
"""
import numpy as np


def _dist():
    import torch.distributed as dist
    return dist if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1 else None


def _device(dist):
    return "cuda" if dist.get_backend() == "nccl" else "cpu"


def scene_seed(base, rank, index, stride=100):
    """Seed of scene `index` of `rank` when every rank makes its own scenes."""
    return base + stride * rank + index


def partition_by_cost(costs, world):
    """Split items of the given costs over `world` ranks, largest first onto
    the least-loaded rank (longest-processing-time rule).  Returns one sorted
    index list per rank; every rank computing it gets the same answer."""
    costs = [float(c) for c in costs]
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    load = [0.0] * world
    parts = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        parts[r].append(i)
        load[r] += costs[i]
    return [sorted(p) for p in parts]


def barrier():
    dist = _dist()
    if dist is not None:
        dist.barrier()


def max_over_ranks(value):
    """The largest of every rank's value (the job ends with its slowest rank)."""
    dist = _dist()
    if dist is None:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=_device(dist))
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value):
    """The sum of every rank's value (the work the whole job did)."""
    dist = _dist()
    if dist is None:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=_device(dist))
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def whole_job_rate(units, seconds):
    """Units all ranks processed per second of the slowest rank."""
    return sum_over_ranks(units) / max_over_ranks(seconds)


def balance(costs, parts):
    """Largest rank load over the mean load of a partition (1 = perfect)."""
    loads = np.array([sum(costs[i] for i in p) for p in parts], np.float64)
    return float(loads.max() / max(loads.mean(), 1e-300))
