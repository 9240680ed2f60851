"""Replica scaling across GPUs: independent work units (facets x output
channels x requests) are dealt round-robin to ranks, each rank runs them on its
own GPU with no data-path collective, and the step time is the maximum over
ranks (a barrier and one MAX all-reduce of a scalar)."""


def shard_units(n_units, rank, world):
    """Unit indices owned by `rank` (round-robin)."""
    if not (0 <= rank < world):
        raise ValueError("rank out of range")
    return list(range(rank, n_units, world))


def max_over_ranks(value, device=None):
    """Maximum of a float over all ranks of the default process group (the
    value itself when no group is initialised)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(units_per_rank, step_seconds):
    """Whole-job rate: all units of all ranks over the slowest rank's time."""
    return float(sum(units_per_rank)) / float(step_seconds)
