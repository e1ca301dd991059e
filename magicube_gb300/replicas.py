"""Replica runs over several ranks (one process per GPU, no data-path
collective): the path shards by vector-row blocks and by (instance, head), so
every rank runs its own copy of the workload.  The only communication is
timing: a barrier before and after the timed region, and the maximum of the
ranks' times, from which the whole-job throughput is computed.  Works with
any torch.distributed backend (NCCL on GPUs, gloo on CPUs)."""
from __future__ import annotations

import os


class Replicas:
    """World size, rank and the timing collectives of a replica run."""

    def __init__(self, backend: str | None = None):
        import torch.distributed as dist
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self._dist = dist
        if self.world > 1 and not dist.is_initialized():
            dist.init_process_group(backend or "nccl")

    def barrier(self) -> None:
        if self.world > 1:
            self._dist.barrier()

    def max(self, x: float, device=None) -> float:
        """The maximum of x over the ranks."""
        if self.world == 1:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64, device=device)
        self._dist.all_reduce(t, op=self._dist.ReduceOp.MAX)
        return float(t.item())

    def throughput(self, units_per_rank: float, seconds: float, device=None) -> float:
        """Whole-job units per second: the units all ranks processed over the
        slowest rank's time."""
        return units_per_rank * self.world / self.max(seconds, device)

    def close(self) -> None:
        if self.world > 1 and self._dist.is_initialized():
            self._dist.destroy_process_group()
