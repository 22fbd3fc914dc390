"""Replica ranks for multi-GPU runs.

The geometry path has no exchange step: under torchrun every rank rebuilds
its own replica of the world on its own GPU. The only cross-rank operations
are a barrier around the timed region and the maximum of the ranks' timed
milliseconds, from which the whole-job throughput is computed.
"""
import os


def init(backend=None, timeout_s=None):
    """(rank, world_size, torch.distributed or None) from the torchrun
    environment; one process group when WORLD_SIZE > 1. A collective that a
    rank never joins fails after timeout_s (default: the backend's)."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 1, None
    import torch
    import torch.distributed as dist
    rank = int(os.environ.get("RANK", "0"))
    if backend is None:
        backend = "nccl" if torch.cuda.is_available() else "gloo"
    if backend == "nccl":
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    if timeout_s is None:
        dist.init_process_group(backend)
    else:
        import datetime
        dist.init_process_group(backend, timeout=datetime.timedelta(seconds=timeout_s))
    return rank, ws, dist


def max_over_ranks(value, dist, device="cpu"):
    """The largest of every rank's `value` (every rank gets it)."""
    if dist is None:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank, world_size, slowest_ms):
    """Units processed by all ranks per second, timed by the slowest rank."""
    return units_per_rank * world_size / (slowest_ms / 1e3)


def finish(dist):
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
