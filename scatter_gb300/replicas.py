"""Several GPUs: independent replicas, one per process and rank.

The path does not partition one mesh across GPUs: that would need a halo exchange per SpMV
and an all-reduce per PCG dot product.  What shards is independent work: realisations,
meshes and whole solves, one replica per rank with no collective on the data path.  Only the
timing is combined across ranks: a barrier on either side of the timed region, the longest
rank's time, and the units every rank processed.  Works with any torch.distributed backend
(NCCL on GPUs, gloo on CPU).
"""
import torch


def _group():
    import torch.distributed as dist

    return dist if dist.is_available() and dist.is_initialized() else None


def world():
    """(world size, rank); (1, 0) without a process group."""
    dist = _group()
    return (dist.get_world_size(), dist.get_rank()) if dist else (1, 0)


def barrier():
    """Barrier over the ranks (no-op for one rank)."""
    dist = _group()
    if dist and dist.get_world_size() > 1:
        dist.barrier()


def job_rate(ms_local, units_local, device=None):
    """(ms, units per second) of the whole job: the longest rank's ms, and the units all ranks
    processed divided by that time.  `device` holds the reduction tensors (the rank's GPU for
    NCCL, None for gloo)."""
    dist = _group()
    if not dist or dist.get_world_size() == 1:
        return float(ms_local), float(units_local) / (float(ms_local) / 1e3)
    t = torch.tensor([float(ms_local)], dtype=torch.float64, device=device)
    u = torch.tensor([float(units_local)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    ms = float(t.item())
    return ms, float(u.item()) / (ms / 1e3)
