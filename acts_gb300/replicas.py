"""Multi-GPU use of the fitter: replicas only. Tracks and events are
independent (the reference fits them one by one, TrackFittingAlgorithm.cpp
:117-170), so N GPUs run N independent fitters on disjoint shards of the
events with no collective on the data path; the only communication is the
host-side reduction of timings and counts at the end.

    rank, world, local = env()
    mine = shard(event_ids, rank, world)      # disjoint, covering
    ...fit `mine` on cuda:local...
    t = max_over_ranks(local_ms)               # the job's wall time
    n = sum_over_ranks(local_tracks)
"""
import os


def env():
    """(rank, world_size, local_rank) from the torchrun environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def shard(items, rank, world):
    """The items rank `rank` of `world` owns: round-robin, so shards differ
    in size by at most one and together cover every item exactly once."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank %d outside a world of %d" % (rank, world))
    return list(items)[rank::world]


def rank_seed(seed, rank):
    """Seed of a rank's synthetic workload (distinct per rank)."""
    return int(seed) + 1000 * int(rank)


def _reduce(value, op):
    import torch
    import torch.distributed as dist

    if not dist.is_available() or not dist.is_initialized():
        return float(value)
    dev = torch.device("cuda", torch.cuda.current_device()) \
        if dist.get_backend() == "nccl" else torch.device("cpu")
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=op)
    return float(t.item())


def max_over_ranks(value):
    """Maximum of `value` over all ranks (the value itself without a process group)."""
    import torch.distributed as dist

    return _reduce(value, dist.ReduceOp.MAX)


def sum_over_ranks(value):
    """Sum of `value` over all ranks."""
    import torch.distributed as dist

    return _reduce(value, dist.ReduceOp.SUM)
