"""Replica coordination for one process per GPU (the multi-GPU form of this path: no data-path collective).

Every rank solves its own problems; the ranks only meet for a barrier around timed regions, the maximum of their
times and the sum of their counts.  Independent problems (the batched and served forms) are sharded round-robin.
RANK / WORLD_SIZE / LOCAL_RANK / MASTER_ADDR / MASTER_PORT come from the launcher (torchrun); with WORLD_SIZE 1
nothing is initialised.  The backend is NCCL when CUDA is available, gloo otherwise (the CPU tests).
"""
from __future__ import annotations

import os


class Replicas:
    def __init__(self, backend: str | None = None):
        self.rank = int(os.environ.get("RANK", "0"))
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self._td = None
        self._torch = None
        self.device = "cpu"
        if self.world > 1:
            import torch
            import torch.distributed as td

            if backend is None:
                backend = "nccl" if torch.cuda.is_available() else "gloo"
            if backend == "nccl":
                torch.cuda.set_device(self.local)
                self.device = "cuda"
            td.init_process_group(backend)
            self._td, self._torch = td, torch

    def barrier(self):
        if self._td:
            self._td.barrier()
            if self.device == "cuda":
                self._torch.cuda.synchronize()

    def _reduce(self, x: float, op) -> float:
        t = self._torch.tensor([float(x)], dtype=self._torch.float64, device=self.device)
        self._td.all_reduce(t, op=op)
        return float(t.item())

    def max(self, x: float) -> float:
        return self._reduce(x, self._td.ReduceOp.MAX) if self._td else float(x)

    def sum(self, x: float) -> float:
        return self._reduce(x, self._td.ReduceOp.SUM) if self._td else float(x)

    def shard(self, items):
        """This rank's share of independent problems (round-robin, so sizes spread evenly)."""
        return list(items)[self.rank::self.world]

    def close(self):
        if self._td:
            self._td.destroy_process_group()
            self._td = None
