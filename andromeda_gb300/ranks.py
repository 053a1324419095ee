"""Host logic of multi-GPU runs: one process per GPU, no collective on the
data path.

The reference distributes its dense rows over MPI ranks (mod_plis.f90); here a
single body's system fits one GB300, so

* a single-body workload runs one independent solve per rank (replicas);
* the batched workload shards by body: rank r solves bodies i with
  i % world == r (weak scaling, every rank a disjoint share);
* the job's time is the slowest rank's: a max over ranks of the per-rank
  device time, after a barrier on both sides of the timed region.

The only collectives are the barrier and that max (torch.distributed; NCCL on
GPUs, gloo in the CPU tests).
"""
import os


def dist_env():
    """(rank, world, local rank) from the torchrun environment (1 process: 0, 1, 0)."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


def shard(n, world, rank):
    """Indices of the bodies rank `rank` of `world` solves: i % world == rank."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"bad rank {rank} of {world}")
    return list(range(rank, n, world))


def _dist():
    import torch.distributed as dist
    return dist if dist.is_available() and dist.is_initialized() else None


def barrier():
    d = _dist()
    if d is not None:
        d.barrier()


def max_over_ranks(values, device="cpu"):
    """Element-wise max of a list of floats over all ranks (identity without a
    process group).  `device`: where the reduction tensor lives ("cuda" for
    NCCL, "cpu" for gloo)."""
    d = _dist()
    vals = [float(v) for v in values]
    if d is None or d.get_world_size() == 1:
        return vals
    import torch
    t = torch.tensor(vals, dtype=torch.float64, device=device)
    d.all_reduce(t, op=d.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]
