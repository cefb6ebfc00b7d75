"""Multi-GPU form of the raycaster: replicas only.

Views (and serving requests) are independent, so N GPUs each hold their own
brick pool and render a disjoint share of the views; framebuffers return to
the host from each GPU independently.  There is no data exchange between
ranks; the only collectives are the benchmark's barrier and the max over
ranks of the timed region.
"""


def shard(n_items, rank, world):
    """Contiguous, balanced share of n_items for `rank` of `world` (sizes
    differ by at most one; every item is owned exactly once)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    base, extra = divmod(n_items, world)
    start = rank * base + min(rank, extra)
    return list(range(start, start + base + (1 if rank < extra else 0)))
