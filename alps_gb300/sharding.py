"""Replica sharding of independent evaluation units (map lattice points,
root solves, k-steps) over ranks.  Units are independent, so ranks exchange
nothing while computing; only the final gather for reporting uses a
collective."""


def shard_range(n, rank, world):
    """Contiguous block [lo, hi) of n units owned by rank (sizes differ by at
    most one; lower ranks get the extra units)."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError("bad rank/world")
    base, rem = divmod(n, world)
    lo = rank * base + min(rank, rem)
    hi = lo + base + (1 if rank < rem else 0)
    return lo, hi
