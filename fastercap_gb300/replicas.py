"""Job-level parallelism over several GPUs: one process per GPU, each an
independent replica of the solver (a geometry never spans GPUs, so there is
no data-path collective). The only exchanges are host-side bookkeeping: a
barrier around timed regions, the maximum of the ranks' times, and the
assignment of independent jobs (geometries, requests) to ranks.

Works with the NCCL backend (CUDA tensors) on GPU nodes and with gloo (CPU
tensors) in the multi-process tests.
"""

from __future__ import annotations

import os


def dist_env() -> tuple[int, int, int]:
    """(rank, world size, local rank) from the torchrun environment."""
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def _device():
    import torch
    import torch.distributed as dist
    if dist.get_backend() == "nccl":
        return torch.device("cuda", torch.cuda.current_device())
    return torch.device("cpu")


def barrier(world: int) -> None:
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(values, world: int) -> list:
    """Element-wise maximum of a list of floats over all ranks."""
    vals = [float(v) for v in values]
    if world <= 1:
        return vals
    import torch
    import torch.distributed as dist
    t = torch.tensor(vals, dtype=torch.float64, device=_device())
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t.cpu()]


def sum_over_ranks(values, world: int) -> list:
    vals = [float(v) for v in values]
    if world <= 1:
        return vals
    import torch
    import torch.distributed as dist
    t = torch.tensor(vals, dtype=torch.float64, device=_device())
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return [float(x) for x in t.cpu()]


def shard(n_jobs: int, rank: int, world: int) -> list:
    """Jobs of this rank: job j runs on rank j mod world (round robin keeps
    the ranks' shares of a size-sorted or random job list alike)."""
    return list(range(rank, n_jobs, world))


def throughput(units_per_rank: float, world: int, seconds_max: float) -> float:
    """Whole-job throughput: every rank processed units_per_rank units; the
    job took as long as the slowest rank."""
    return world * units_per_rank / seconds_max


def gather_to_all(obj, world: int) -> list:
    """Every rank's picklable obj, in rank order, on every rank."""
    if world <= 1:
        return [obj]
    import torch.distributed as dist
    out = [None] * world
    dist.all_gather_object(out, obj)
    return out
