"""Replica runs on one node: one process per GPU, each counting its own copy of
the workload.  The path's inputs are independent byte streams, so ranks share
no data and no collective runs on the data path; the group only lines up the
timed region (barrier) and reduces the per-rank figures, as a ``torchrun``
launch expects: whole-job throughput = units of all ranks / the slowest
rank's time.

Any ``torch.distributed`` backend works: nccl on GPUs, gloo on the CPU.
Rendezvous comes from the environment torchrun sets (RANK, LOCAL_RANK,
WORLD_SIZE, MASTER_ADDR, MASTER_PORT).
"""
from __future__ import annotations

import os


def env() -> tuple[int, int, int]:
    """(world size, rank, local rank) from the launcher's environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


class ReplicaGroup:
    def __init__(self, backend: str = "nccl"):
        self.world, self.rank, self.local = env()
        self.backend = backend
        self._owned = False
        if self.world > 1:
            import torch.distributed as dist
            if not dist.is_initialized():
                dist.init_process_group(backend)
                self._owned = True

    def _tensor(self, v: float):
        import torch
        dev = "cuda" if self.backend == "nccl" else "cpu"
        return torch.tensor([float(v)], dtype=torch.float64, device=dev)

    def barrier(self, sync_device: bool = True) -> None:
        if self.world > 1:
            import torch.distributed as dist
            dist.barrier()
        if sync_device:
            import torch
            if torch.cuda.is_available():
                torch.cuda.synchronize()

    def _reduce(self, v: float, op: str) -> float:
        if self.world == 1:
            return float(v)
        import torch.distributed as dist
        t = self._tensor(v)
        dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
        return float(t.item())

    def max_over_ranks(self, v: float) -> float:
        return self._reduce(v, "max")

    def sum_over_ranks(self, v: float) -> float:
        return self._reduce(v, "sum")

    def throughput(self, units: float, ms: float) -> float:
        """Units of all ranks per second over the slowest rank's time."""
        return self.sum_over_ranks(units) / (self.max_over_ranks(ms) * 1e-3)

    def close(self) -> None:
        if self._owned:
            import torch.distributed as dist
            dist.destroy_process_group()
            self._owned = False
