"""Multi-GPU form of the lensing path: independent replicas, one process per
GPU (torchrun), no collective on the data path.  Each rank solves its own
requests (its own seeds); the only communication is a barrier around the timed
region and a max-reduction of the per-rank elapsed time, so the whole-job
throughput is (ranks x solves per rank) / slowest rank (weak scaling).

The backend is NCCL on GPUs; the host logic also runs on gloo (CPU tests)."""
from __future__ import annotations

import os

import torch
import torch.distributed as dist


class Replicas:
    def __init__(self, backend: str | None = None):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.backend = backend or ("nccl" if torch.cuda.is_available() else "gloo")
        self.owns_group = False
        if self.world > 1 and not dist.is_initialized():
            if self.backend == "nccl":
                torch.cuda.set_device(self.local)
            dist.init_process_group(self.backend)
            self.owns_group = True

    @property
    def device(self):
        if self.backend == "nccl":
            return torch.device("cuda", self.local if self.world > 1 else 0)
        return torch.device("cpu")

    def seed(self, base: int) -> int:
        """Per-rank seed: every replica solves different requests."""
        return base + 17 * self.rank

    def barrier(self):
        if self.world > 1:
            dist.barrier()

    def max(self, x: float) -> float:
        """Maximum of a per-rank scalar over all ranks (the slowest replica)."""
        if self.world == 1:
            return float(x)
        t = torch.tensor([float(x)], dtype=torch.float64, device=self.device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    def throughput(self, units_per_rank: float, seconds: float) -> float:
        """Whole-job units per second: all ranks' units over the slowest rank's time."""
        return self.world * units_per_rank / self.max(seconds)

    def close(self):
        if self.owns_group and dist.is_initialized():
            dist.destroy_process_group()
