"""Independent replicas on several GPUs (one process per GPU, torchrun).

The standalone solves and the ensemble's members are independent, so N GPUs
run N replicas: each rank draws its own seeds, no data crosses ranks during a
step, and a measurement is the work of all ranks over the slowest rank's time.
Works with any initialised torch.distributed backend (NCCL on GPUs, gloo on CPU).
"""
import torch


def seeds_for_rank(rank, count, stride=1000):
    """Seeds of one rank's inputs; disjoint across ranks for count <= stride."""
    if count > stride:
        raise ValueError("count %d exceeds the per-rank seed stride %d" % (count, stride))
    return [stride * int(rank) + s for s in range(int(count))]


def _dist():
    import torch.distributed as dist
    return dist if dist.is_available() and dist.is_initialized() else None


def max_over_ranks(value, device=None):
    """Maximum of a float over all ranks (the value itself without a process group)."""
    dist = _dist()
    if dist is None:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(units_per_rank, world, slowest_seconds):
    """Whole-job throughput: the units of all ranks over the slowest rank's time."""
    if not slowest_seconds > 0:
        raise ValueError("slowest_seconds must be positive")
    return units_per_rank * world / slowest_seconds
