"""Sharding a batch of independent sections over ranks (one GPU each).

The sections of a batch share nothing, so a multi-GPU run splits them with
no data-path exchange: each rank processes its own subset in one batched
launch sequence.  The split balances samples (the work is proportional to
them) and is deterministic, so every rank computes the same plan alone.
"""


def shard_sections(shapes, rank, world):
    """Indices of the sections (by position in `shapes`) assigned to `rank`
    of `world`: largest first, each to the rank with the fewest samples so
    far (lowest rank on ties).  Returned in ascending order."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a world of {world}")
    sizes = []
    for k, sh in enumerate(shapes):
        n = 1
        for d in sh:
            n *= int(d)
        sizes.append((n, k))
    load = [0] * world
    mine = []
    for n, k in sorted(sizes, key=lambda t: (-t[0], t[1])):
        r = min(range(world), key=lambda i: (load[i], i))
        load[r] += n
        if r == rank:
            mine.append(k)
    return sorted(mine)
