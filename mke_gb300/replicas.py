"""Replicas across the GPUs of one node.

A trajectory does not shard at these sizes: every Krylov step of its solves
reduces over the whole mesh.  N processes (one per GPU, launched by torchrun:
RANK / WORLD_SIZE / LOCAL_RANK) therefore run independent trajectories, or
independent slices of an ensemble or of a request stream, with no collective
on the data path.  The only collectives are for bookkeeping: the maximum of
the per-rank timings (whole-job throughput = all ranks' units / the slowest
rank's time) and, for an ensemble, rank 0 gathering the members' results on
the host.  The backend is NCCL on GPUs and gloo for the CPU tests.
"""
from __future__ import annotations

import os

import numpy as np


def env():
    """(world size, rank, local rank) from the launcher's environment (1, 0, 0 alone)."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def shard(n: int, rank: int, world: int):
    """The [start, stop) slice of n independent units owned by `rank`: contiguous,
    in rank order, sizes differing by at most one."""
    if world < 1 or not 0 <= rank < world or n < 0:
        raise ValueError("bad shard arguments")
    base, extra = divmod(n, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def init(backend: str, device=None) -> bool:
    """Join the process group when launched with more than one rank; returns
    whether a group exists.  device: the rank's CUDA device (NCCL)."""
    world, _, _ = env()
    if world <= 1:
        return False
    import torch.distributed as dist
    if not dist.is_initialized():
        if device is not None:
            dist.init_process_group(backend, device_id=device)
        else:
            dist.init_process_group(backend)
    return True


def barrier():
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.barrier()


def max_over_ranks(values, device=None):
    """Element-wise maximum of a list of floats over the ranks (the values
    themselves when alone)."""
    import torch
    import torch.distributed as dist
    vals = [float(v) for v in values]
    if not (dist.is_available() and dist.is_initialized()):
        return vals
    t = torch.tensor(vals, dtype=torch.float64, device=device if device is not None else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t.cpu().tolist()]


def gather_rows(local: np.ndarray):
    """Rank 0 receives the ranks' row blocks concatenated in rank order (the
    ensemble in member order when the blocks come from shard()); other ranks
    get None.  Alone: the block itself."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return local
    world, rank = dist.get_world_size(), dist.get_rank()
    parts = [None] * world if rank == 0 else None
    dist.gather_object(np.ascontiguousarray(local), parts, dst=0)
    if rank != 0:
        return None
    return np.concatenate(parts, axis=0)


def whole_job_rate(units_per_rank: float, seconds_max: float, world: int) -> float:
    """Throughput of the whole job: every rank's units over the slowest rank's time."""
    return world * units_per_rank / seconds_max if seconds_max > 0 else 0.0


def finish():
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.destroy_process_group()
