"""Ensemble members spread over GPUs: one process per GPU, no data-path collective.

GPU Ocean's only parallelism is MPI ranks that each own a range of ensemble
members (E/MPIOceanModelEnsemble.py:133, E/ = src/gpuocean/ensembles); members
are independent between observations.  Here each rank drives its own batched
engine on its own GPU.  The host needs two things across ranks: a contiguous
member range per rank, and - for throughput figures - a barrier and a maximum
of the ranks' wall times (the job is as fast as its slowest rank).  This
module provides both over ``torch.distributed`` (NCCL between GPUs, gloo on
CPU).  With one rank every call is local.
"""
from __future__ import annotations

import os


def member_range(n_members, rank, world):
    """Contiguous member range [first, first + count) of `rank` out of
    `world` ranks; the first n_members % world ranks get one member more."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a world of {world}")
    base, extra = divmod(int(n_members), int(world))
    first = rank * base + min(rank, extra)
    return first, base + (1 if rank < extra else 0)


def env_ranks():
    """(rank, world, local rank) from the torchrun environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


class ReplicaGroup:
    """Barrier and reductions across the ranks of one job (a no-op for one
    rank).  backend: "nccl" between GPUs, "gloo" on CPU."""

    def __init__(self, world=None, backend="gloo", rank=None):
        r, w, _ = env_ranks()
        self.world = w if world is None else int(world)
        self.rank = r if rank is None else int(rank)
        self.td = None
        if self.world > 1:
            import torch.distributed as td
            if not td.is_initialized():
                td.init_process_group(backend=backend, rank=self.rank, world_size=self.world)
            self.td = td

    def barrier(self):
        if self.td is not None:
            self.td.barrier()

    def _reduce(self, v, op):
        if self.td is None:
            return float(v)
        import torch
        t = torch.tensor([float(v)], dtype=torch.float64)
        if self.td.get_backend() == "nccl":
            t = t.cuda()
        self.td.all_reduce(t, op=op)
        return float(t.item())

    def max(self, v):
        return self._reduce(v, None if self.td is None else self.td.ReduceOp.MAX)

    def sum(self, v):
        return self._reduce(v, None if self.td is None else self.td.ReduceOp.SUM)

    def throughput(self, local_units, local_seconds):
        """Whole-job rate: all ranks' units over the slowest rank's time."""
        return self.sum(local_units) / self.max(local_seconds)

    def close(self):
        if self.td is not None and self.td.is_initialized():
            self.td.destroy_process_group()
        self.td = None
