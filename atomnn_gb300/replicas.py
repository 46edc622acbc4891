"""Replica distribution of structures over GPUs (one process per GPU).

Structures are independent units, so N GPUs evaluate disjoint blocks of a structure list with no
collective on the data path.  The block split follows the reference's own distribution of whole
structures over MPI ranks (thread::Dist, src/thread/dist.hpp:21-53, used by src/nnp/nnpce.cpp:222):
rank r gets a contiguous block, the first (n mod world) ranks one structure more.
"""


def shard(n, rank, world):
    """(offset, count) of rank's block of n structures."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError("invalid rank/world")
    base, extra = divmod(n, world)
    count = base + (1 if rank < extra else 0)
    offset = rank * base + min(rank, extra)
    return offset, count


def gather_results(local, group=None):
    """Concatenate per-rank result lists in rank order (torch.distributed all_gather_object)."""
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized():
        return list(local)
    out = [None] * dist.get_world_size(group)
    dist.all_gather_object(out, list(local), group=group)
    return [x for part in out for x in part]
