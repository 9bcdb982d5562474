"""Independent replicas of the engine on several GPUs of one node.

The interaction path shards naturally (walks are independent given their
lists), but this module runs one GPU per process without exchanging particles:
each rank evolves its own system (seeded by its rank), and the job's
throughput is the work of all ranks over the slowest rank's time.  The only
collectives are these scalar reductions and barriers (NCCL between GPUs,
gloo for the CPU tests of the same logic).
"""
import os


def rank_info():
    """(world size, rank, local rank) from the launcher's environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def init(backend, device=None):
    """Joins the process group when there is more than one rank; returns the
    world size."""
    world, _, _ = rank_info()
    if world > 1:
        import torch.distributed as dist
        if not dist.is_initialized():
            if device is not None:
                dist.init_process_group(backend, device_id=device)
            else:
                dist.init_process_group(backend)
    return world


def barrier():
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.barrier()


def _reduce(value, op, device):
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=op)
    return float(t.item())


def reduce_max(value, device="cpu"):
    import torch.distributed as dist
    return _reduce(value, dist.ReduceOp.MAX, device)


def reduce_sum(value, device="cpu"):
    import torch.distributed as dist
    return _reduce(value, dist.ReduceOp.SUM, device)


def aggregate_rate(units, ms, steps, device="cpu"):
    """(job rate, max ms): units summed over the ranks x steps / slowest
    rank's time."""
    total = reduce_sum(units, device)
    worst = reduce_max(ms, device)
    return total * steps / (worst * 1e-3), worst


def replica_seed(base, rank):
    return int(base) + int(rank)


def finalize():
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.destroy_process_group()
