"""Ensemble sharding across ranks: independent instances, no exchange.

The reference decomposes one lattice into MPI subdomains with halo layers
(Subdomain.cpp:67-230, Simulation.cpp:202-872).  Here one lattice stays on
one GPU; what spreads over GPUs is an ensemble of independent vessels
(lbm_batch_create per rank), so no data crosses ranks during the steps.
Every rank computes the same partition from the same per-instance weights
(fluid node counts), so the partition itself needs no communication.
"""


def partition(weights, nranks):
    """Instance indices of each rank: longest-processing-time greedy (heaviest
    instance first, to the least loaded rank, ties to the lowest rank); each
    list in ascending order.  Every instance is assigned exactly once."""
    if nranks < 1:
        raise ValueError("nranks must be >= 1")
    load = [0] * nranks
    out = [[] for _ in range(nranks)]
    for i in sorted(range(len(weights)), key=lambda k: (-weights[k], k)):
        r = min(range(nranks), key=lambda k: (load[k], k))
        out[r].append(i)
        load[r] += weights[i]
    return [sorted(x) for x in out]


def shard(weights, rank, nranks):
    """Instance indices of `rank` (see partition)."""
    return partition(weights, nranks)[rank]
