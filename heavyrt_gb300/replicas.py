"""Replicas across GPUs: one process per GPU, each tracing its own full copy of
the workload (rays are independent, so no collective is needed on the data
path).  This module holds the host-side coordination the benchmark uses:
process-group set-up from the torchrun environment, barriers around the
timed region, the slowest rank's time, and the whole-job throughput.

Works with any torch.distributed backend: NCCL between GPUs, gloo on CPU
(the tests run two gloo ranks).
"""
from __future__ import annotations

import os
from dataclasses import dataclass


@dataclass
class Rank:
    rank: int
    world: int
    local: int

    @property
    def leader(self) -> bool:
        return self.rank == 0


def from_env() -> Rank:
    """RANK / WORLD_SIZE / LOCAL_RANK as torchrun sets them (one process when absent)."""
    return Rank(int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
                int(os.environ.get("LOCAL_RANK", "0")))


def init(r: Rank, backend: str = "nccl"):
    """Joins the process group when there is more than one rank."""
    if r.world > 1:
        import torch.distributed as dist

        if not dist.is_initialized():
            dist.init_process_group(backend)


def barrier(r: Rank):
    if r.world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(r: Rank, value: float, device: str = "cpu") -> float:
    """The largest value over all ranks (the job's step takes its slowest rank's time)."""
    if r.world == 1:
        return float(value)
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(r: Rank, units_per_rank: float, ms_per_step_max: float) -> float:
    """Whole-job rate in units per second: every rank processes units_per_rank
    per step (weak scaling) and a step takes the slowest rank's time."""
    return r.world * units_per_rank / (ms_per_step_max * 1e-3)


def finish(r: Rank):
    if r.world > 1:
        import torch.distributed as dist

        if dist.is_initialized():
            dist.destroy_process_group()
