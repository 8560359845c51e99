"""Independent replicas, one per rank, for running the benchmark on several
GPUs of a node.

A state vector that fits one GPU has nothing to exchange with another: every
rank runs its own circuit (its own seed) on its own GPU, and the only
collectives are the barriers around the timed region and the reduction of
the results.  The job's throughput is all ranks' units over the slowest
rank's time.

Under torchrun the rank comes from RANK / WORLD_SIZE / LOCAL_RANK; without
them this is a single rank and makes no collective call.
"""
from __future__ import annotations

import os


class Replicas:
    def __init__(self, backend: str | None = None):
        self.rank = int(os.environ.get("RANK", "0"))
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.backend = backend or "nccl"
        self.dist = None
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group(self.backend)
            self.dist = dist

    @property
    def leader(self) -> bool:
        return self.rank == 0

    def seed(self, base: int) -> int:
        """A different circuit on every rank."""
        return base + self.rank

    def barrier(self) -> None:
        if self.dist:
            self.dist.barrier()

    def _reduce(self, x: float, op_name: str) -> float:
        if not self.dist:
            return float(x)
        import torch
        dev = "cuda" if self.backend == "nccl" else "cpu"
        t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
        self.dist.all_reduce(t, op=getattr(self.dist.ReduceOp, op_name))
        return float(t.item())

    def max(self, x: float) -> float:
        return self._reduce(x, "MAX")

    def sum(self, x: float) -> float:
        return self._reduce(x, "SUM")

    def gather(self, obj) -> list:
        """Every rank's `obj` (any picklable value), in rank order, on every
        rank: one all-gather, outside any timed region."""
        if not self.dist:
            return [obj]
        out = [None] * self.world
        self.dist.all_gather_object(out, obj)
        return out

    def throughput(self, units: float, seconds: float) -> float:
        """All ranks' units over the slowest rank's seconds."""
        return self.sum(units) / self.max(seconds)

    def close(self) -> None:
        if self.dist:
            self.dist.barrier()
            self.dist.destroy_process_group()
            self.dist = None
