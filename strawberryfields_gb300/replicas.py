"""Multi-GPU use of the simulator: independent replicas, no data-path
collective.  Each rank simulates its own circuits on its own GPU; the only
exchange is the reduction of per-rank timings for whole-job throughput."""


def job_throughput(local_ms, units_per_rank, group=None):
    """Whole-job units/s from each rank's elapsed milliseconds: the slowest
    rank's time bounds the job (max over ranks), every rank contributes
    ``units_per_rank`` units.  Works with any torch.distributed backend
    (gloo on CPU, nccl on GPUs); returns (units_per_s, max_ms)."""
    import torch
    import torch.distributed as dist

    if not dist.is_available() or not dist.is_initialized():
        return units_per_rank / (local_ms / 1e3), local_ms
    backend = dist.get_backend(group)
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    t = torch.tensor([float(local_ms)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    world = dist.get_world_size(group)
    max_ms = float(t.item())
    return world * units_per_rank / (max_ms / 1e3), max_ms
