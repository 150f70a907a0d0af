"""Replica bookkeeping for `bench.py --gpus N`: the path does not shard (every box has one GPU and
the spec workload fits one), so N ranks run N independent replicas; the job time is the
maximum over ranks and the throughput counts every rank's DoF."""


def max_over_ranks(value, group=None):
    """Maximum of a float over all ranks (works with the gloo and nccl backends)."""
    import torch
    import torch.distributed as dist

    if not dist.is_available() or not dist.is_initialized():
        return float(value)
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())


def job_throughput(units_per_rank, seconds_per_step_max, world_size):
    """Whole-job throughput: units processed by all ranks per (slowest rank's) step time."""
    return world_size * units_per_rank / seconds_per_step_max
