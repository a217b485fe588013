"""Replicas on several GPUs of one node: every rank serves its own requests on
its own GPU (no data-path collective -- instances are independent, so the
path shards by request).  Only the measurement crosses ranks: a barrier
before and after the timed region and the maximum of the ranks' times, from
which the whole job's throughput follows.

Launched one process per GPU (``torch.distributed.run``); RANK, LOCAL_RANK
and WORLD_SIZE come from the environment.
"""

from __future__ import annotations

import os

import torch


def world() -> tuple:
    """(rank, local rank, world size) from the launcher's environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0")),
            int(os.environ.get("WORLD_SIZE", "1")))


def init(backend: str = "nccl") -> None:
    """Join the process group when there is more than one rank (nccl binds
    this rank's GPU; gloo runs on the CPU)."""
    import torch.distributed as dist

    _, local, size = world()
    if size > 1 and not dist.is_initialized():
        if backend == "nccl":
            dist.init_process_group("nccl", device_id=torch.device("cuda", local))
        else:
            dist.init_process_group(backend)


def barrier() -> None:
    import torch.distributed as dist

    if dist.is_initialized() and dist.get_world_size() > 1:
        dist.barrier()


def max_over_ranks(value: float) -> float:
    """The largest of the ranks' values (every rank receives it)."""
    import torch.distributed as dist

    if not (dist.is_initialized() and dist.get_world_size() > 1):
        return float(value)
    dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend() == "nccl" else torch.device("cpu")
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank: float, seconds: float) -> tuple:
    """(whole-job units/s, max-over-ranks seconds): every rank processed
    units_per_rank in its own seconds; the job took the slowest rank's time."""
    import torch.distributed as dist

    size = dist.get_world_size() if dist.is_initialized() else 1
    t = max_over_ranks(seconds)
    return size * units_per_rank / t, t


def finish() -> None:
    import torch.distributed as dist

    if dist.is_initialized():
        dist.destroy_process_group()
