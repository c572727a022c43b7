"""Replicas across GPUs (one process per GPU, no data-path collective).

Frames and views are independent, so the multi-GPU form of this path is N
replicas: each rank renders its own views; the only cross-rank traffic is
host bookkeeping -- which views a rank takes, and the slowest rank's time for
throughput figures.  These helpers work with any torch.distributed backend
(gloo on CPU, NCCL on GPUs).
"""
import torch


def _dist():
    import torch.distributed as dist
    return dist if dist.is_available() and dist.is_initialized() else None


def world():
    d = _dist()
    return (d.get_world_size(), d.get_rank()) if d else (1, 0)


def partition_views(nviews, nranks, rank):
    """Contiguous, balanced slice of view indices for `rank` (sizes differ by
    at most one)."""
    base, extra = divmod(nviews, nranks)
    start = rank * base + min(rank, extra)
    return list(range(start, start + base + (1 if rank < extra else 0)))


def max_over_ranks(x):
    """The largest x over all ranks (x itself without a process group)."""
    d = _dist()
    if d is None:
        return float(x)
    dev = 'cuda' if d.get_backend() == 'nccl' else 'cpu'
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    d.all_reduce(t, op=d.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x):
    d = _dist()
    if d is None:
        return float(x)
    dev = 'cuda' if d.get_backend() == 'nccl' else 'cpu'
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    d.all_reduce(t, op=d.ReduceOp.SUM)
    return float(t.item())


def aggregate_rate(units_this_rank, seconds_this_rank):
    """Whole-job throughput: all ranks' units over the slowest rank's time."""
    return sum_over_ranks(units_this_rank) / max_over_ranks(seconds_this_rank)
