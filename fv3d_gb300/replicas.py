"""Multi-GPU runs as independent replicas.

Every problem of this code fits one GPU, and a batch splits by problem with
no exchange at all, so N GPUs run N independent replicas (one process per
GPU, launched by torchrun): there is no collective on the data path.  The
only communication is in the measurement -- a barrier around the timed
region and a max over ranks of the elapsed time -- so the aggregate
throughput is (work of all ranks) / (slowest rank's time).
"""
import os


def dist_info():
    """(world_size, rank, local_rank) from the torchrun environment."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def init(backend):
    """Joins the process group when running under torchrun (world > 1)."""
    world, rank, local = dist_info()
    if world > 1:
        import torch.distributed as dist
        if not dist.is_initialized():
            dist.init_process_group(backend)
    return world, rank, local


def barrier():
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.barrier()


def max_over_ranks(value, device="cpu"):
    """Largest `value` over all ranks (the value itself when alone)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(units_per_rank, world, local_seconds, device="cpu"):
    """Whole-job rate: units of all ranks over the slowest rank's time."""
    slowest = max_over_ranks(local_seconds, device)
    return units_per_rank * world / slowest, slowest


def shutdown():
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.destroy_process_group()
