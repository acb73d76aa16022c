"""Multi-rank helpers (one process per GPU, launched by torchrun).

Particles and error seeds are independent, so ranks never exchange data on
the tracking path: each rank takes a contiguous block of seeds (or its own
beam), and the only collective is the max of the per-rank timings.
"""


def shard(n, rank, world):
    """Contiguous block [start, stop) of n items for ``rank`` of ``world``;
    the first n % world ranks get one extra item."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f'rank {rank} of {world}')
    base, extra = divmod(n, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def beam_seed(rank, base=2):
    """RNG seed of a rank's beam in weak-scaling runs."""
    return base + rank


def max_over_ranks(value, device=None):
    """Max of a float over all ranks (identity without torch.distributed)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64,
                     device=device if device is not None else 'cpu')
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
