"""Replica execution across GPUs of one node: one process per GPU, each rendering its own copy of the
workload on its own queue, with no data exchanged between ranks.  A frame of this path does not shard
without an image-gather step that nothing here needs, so multi-GPU runs are replicas; the only
collectives are the timing barrier and the max-over-ranks reduction of the step time.

Used by bench.py under torchrun (NCCL) and by the CPU tests (gloo)."""
import os
from dataclasses import dataclass


@dataclass
class Rank:
    rank: int
    world: int
    local: int

    @property
    def leader(self):
        return self.rank == 0


def from_env():
    """rank, world size and local rank from the torchrun environment (1 process when absent)"""
    return Rank(int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
                int(os.environ.get("LOCAL_RANK", "0")))


def init(r, backend, device=None):
    """join the process group when there is more than one rank"""
    if r.world > 1:
        import torch.distributed as dist
        if device is not None:
            dist.init_process_group(backend, device_id=device)
        else:
            dist.init_process_group(backend)


def barrier(r):
    if r.world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(r, value, device="cpu"):
    """the largest `value` over all ranks (every rank gets it)"""
    if r.world == 1:
        return float(value)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(r, units_per_rank, max_ms):
    """whole-job throughput: the units all ranks processed (each rank the same replica workload) divided
    by the slowest rank's time; per second"""
    return units_per_rank * r.world / (max_ms / 1e3)


def finish(r):
    if r.world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
