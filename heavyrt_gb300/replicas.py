"""Ray work across GPUs: one process per GPU, each either tracing its own full
copy of the workload (replicas, weak scaling) or its contiguous share of one
ray batch (partition, strong scaling) with the results gathered on the host.
Rays are independent, so no collective is needed on the data path.  This
module holds the host-side coordination the benchmark uses: process-group
set-up from the torchrun environment, barriers around the timed region, the
slowest rank's time, the whole-job throughput, the partition of a batch and
the host gather of its results.

Works with any torch.distributed backend: NCCL between GPUs, gloo on CPU
(the tests run two gloo ranks).
"""
from __future__ import annotations

import os
from dataclasses import dataclass

import numpy as np


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


def partition(n: int, r: Rank, align: int = 1) -> tuple[int, int]:
    """Rank r's contiguous share [start, end) of n items, cut at multiples of
    `align` items (whole image bands, say); the shares cover [0, n) in rank
    order and differ by at most one block."""
    if align < 1:
        raise ValueError("align must be positive")
    blocks = (n + align - 1) // align
    base, extra = divmod(blocks, r.world)
    b0 = r.rank * base + min(r.rank, extra)
    b1 = b0 + base + (1 if r.rank < extra else 0)
    return min(n, b0 * align), min(n, b1 * align)


def host_group(r: Rank):
    """A gloo process group for gathers through host memory (NCCL moves device
    tensors only); None for one rank.  Every rank calls it, in the same order."""
    if r.world == 1:
        return None
    import torch.distributed as dist

    return dist.new_group(backend="gloo")


def gather_rows(r: Rank, local: np.ndarray, group=None):
    """Every rank's rows (axis 0; same dtype and row shape everywhere)
    concatenated in rank order on rank 0, through host memory; None on the
    other ranks.  One rank: `local` itself."""
    if r.world == 1:
        return local
    import torch
    import torch.distributed as dist

    a = np.ascontiguousarray(local)
    row_bytes = a.dtype.itemsize * int(np.prod(a.shape[1:], dtype=np.int64))
    counts = torch.tensor([a.shape[0]], dtype=torch.int64)
    all_counts = [torch.zeros(1, dtype=torch.int64) for _ in range(r.world)]
    dist.all_gather(all_counts, counts, group=group)
    sizes = [int(c.item()) for c in all_counts]
    width = max(sizes) * row_bytes
    buf = torch.zeros(width, dtype=torch.uint8)
    if a.size:
        buf[: a.nbytes] = torch.from_numpy(a.reshape(-1).view(np.uint8))
    outs = [torch.zeros(width, dtype=torch.uint8) for _ in range(r.world)] if r.leader else None
    dist.gather(buf, outs, dst=0, group=group)
    if not r.leader:
        return None
    parts = [o.numpy()[: k * row_bytes].view(a.dtype).reshape((k,) + a.shape[1:]) for o, k in zip(outs, sizes)]
    return np.concatenate(parts, axis=0)


def finish(r: Rank):
    if r.world > 1:
        import torch.distributed as dist

        if dist.is_initialized():
            dist.destroy_process_group()
