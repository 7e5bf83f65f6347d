"""Replicas on several GPUs: one independent box per rank, no data exchange.

The path does not shard across GPUs here (one box per GPU, no inter-GPU
collectives), so N GPUs run N replicas of the workload.  The only
collectives are a barrier around the timed region and the maximum of the
ranks' times; throughput is the units all ranks processed divided by the
slowest rank's time (weak scaling).  Ranks come from torchrun's environment
(RANK, LOCAL_RANK, WORLD_SIZE, MASTER_ADDR, MASTER_PORT).
"""

from __future__ import annotations

import os


class Replicas:
    def __init__(self, backend: str | None = None):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.dist = None
        self.backend = backend
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group(backend)
            self.dist = dist

    @property
    def leader(self) -> bool:
        return self.rank == 0

    def barrier(self):
        if self.dist:
            self.dist.barrier()

    def max(self, x: float) -> float:
        """The maximum of x over the ranks (every rank gets it)."""
        if not self.dist:
            return float(x)
        import torch
        dev = f"cuda:{self.local}" if self.backend == "nccl" else "cpu"
        t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def rate(self, units_per_rank: float, seconds: float) -> tuple:
        """(all ranks' units / slowest rank's seconds, slowest seconds)."""
        t = self.max(seconds)
        return units_per_rank * self.world / t, t

    def close(self):
        if self.dist:
            self.dist.destroy_process_group()
            self.dist = None
