"""Replicas across processes: one process per GPU, launched by torch.distributed.run.

A frame does not shard without a triangle broadcast and a tile gather (every raster tile may
need every triangle), and independent scenes need no exchange at all, so N processes render N
independent replicas. The only communication is about timing: a barrier on both sides of a
timed region, the maximum over ranks of its duration, and sums of per-rank rates.
"""
import os


def dist_env():
    """(rank, world size, local rank) from the launcher's environment; (0, 1, 0) when alone."""
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


class Replicas:
    """The process group of a replicated run (none for a single process). `device` is where
    reductions run: "cuda" for NCCL, "cpu" for gloo."""

    def __init__(self, backend="nccl", device="cuda"):
        self.rank, self.world, self.local = dist_env()
        self.device = device
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group(backend)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def _reduce(self, values, op):
        values = [float(v) for v in values]
        if not self.pg:
            return values
        import torch
        t = torch.tensor(values, dtype=torch.float64, device=self.device)
        self.pg.all_reduce(t, op=op(self.pg.ReduceOp))
        return [float(x) for x in t.tolist()]

    def max(self, values):
        """Element-wise maximum over ranks (durations of a timed region, tail latencies)."""
        return self._reduce(values, lambda r: r.MAX)

    def sum(self, values):
        """Element-wise sum over ranks (rates of independent replicas)."""
        return self._reduce(values, lambda r: r.SUM)

    def close(self):
        if self.pg:
            self.pg.barrier()
            self.pg.destroy_process_group()
            self.pg = None
