"""Replica helpers for running independent blocks on several GPUs of one node (one process per
GPU, launched by torch.distributed.run): rank / world / local rank from the environment and
the host-side reductions of per-rank results (timings, counters).  The data path has no
collective: every rank advances its own blocks.  On CPU (tests) the same calls run over gloo.
"""
import os


def dist_env():
    """(rank, world size, local rank) from the torch.distributed.run environment (0, 1, 0 alone)."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def _reduce(value, op):
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=op)
    return float(t.item())


def max_over_ranks(value):
    """Largest value over the ranks (the whole-job time of a replicated step)."""
    import torch.distributed as dist
    return _reduce(value, dist.ReduceOp.MAX)


def sum_over_ranks(value):
    """Sum over the ranks (points or launches of the whole job)."""
    import torch.distributed as dist
    return _reduce(value, dist.ReduceOp.SUM)
