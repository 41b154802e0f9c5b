"""Multi-process plumbing for ``bench.py --gpus N``: one process per GPU.

The force path does not shard here.  ph4 would split j by domain and
allreduce the partial forces (src/amuse_ph4/src/jdata.cc:56-67,
idata.cc:284-313), but this library runs one GPU per process, so N GPUs run
N independent replicas of the same step.  There is no collective on the
data path.  The only communication is a barrier before the timed region and
a max-reduction of the timed seconds, so that the reported whole-job rate is
(units all ranks processed) / (slowest rank's time).

Works with NCCL (GPU ranks) and gloo (CPU ranks, used by the tests).
"""
from __future__ import annotations

import os


def env():
    """(rank, world_size, local_rank) from the torchrun environment."""
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


def init(backend):
    """Join the process group when launched with more than one rank."""
    import torch.distributed as dist
    _, world, _ = env()
    if world > 1 and not dist.is_initialized():
        dist.init_process_group(backend)
    return world


def barrier():
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.barrier()


def max_over_ranks(seconds, device="cpu"):
    """The largest value of ``seconds`` over all ranks (itself with one rank)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(seconds)
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank, world, slowest_seconds):
    """Units all ranks processed per second of the slowest rank."""
    return world * units_per_rank / slowest_seconds


def finalize():
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.destroy_process_group()
