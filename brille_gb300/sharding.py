"""Splitting a query batch across GPUs.

q points are independent, so N GPUs each take a contiguous slice of the
batch with their own copy of the tables; nothing is exchanged on the data
path.
"""


def shard_range(n, rank, world):
    """[start, stop) of rank's slice of n items, sizes differing by ≤ 1."""
    base, extra = divmod(int(n), int(world))
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)
