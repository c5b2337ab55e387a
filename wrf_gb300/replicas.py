"""Host-side logic of the multi-GPU form: independent replicas.

Ensemble members share nothing (no halo, no reduction between them), so N
GPUs advance disjoint subsets of the members with no collective on the data
path.  The only communication is the end-of-run aggregation of the timing:
the whole-job rate is the units all ranks advanced divided by the slowest
rank's time.  One process per GPU (torchrun); the process group is NCCL on
GPUs and gloo for the CPU tests.
"""
import heapq


def shard_members(sizes, world):
    """Size-balanced assignment of members to ranks: longest-processing-time
    greedy (largest member first, to the least-loaded rank).  Returns a list
    of `world` lists of member indices, each sorted; every member appears in
    exactly one list.  Deterministic (ties broken by rank, then index)."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(sizes)), key=lambda q: (-sizes[q], q))
    heap = [(0, r) for r in range(world)]
    out = [[] for _ in range(world)]
    for q in order:
        load, r = heapq.heappop(heap)
        out[r].append(q)
        heapq.heappush(heap, (load + sizes[q], r))
    return [sorted(x) for x in out]


def _reduce(pg, value, op):
    if pg is None:
        return value
    import torch
    dev = "cuda" if pg.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    pg.all_reduce(t, op=op)
    return float(t.item())


def reduce_max(pg, value):
    """Max over ranks (identity without a process group)."""
    if pg is None:
        return value
    return _reduce(pg, value, pg.ReduceOp.MAX)


def reduce_sum(pg, value):
    """Sum over ranks (identity without a process group)."""
    if pg is None:
        return value
    return _reduce(pg, value, pg.ReduceOp.SUM)


def job_rate(pg, local_units, local_seconds):
    """Whole-job throughput: units advanced by all ranks / slowest rank's time."""
    total = reduce_sum(pg, local_units)
    slowest = reduce_max(pg, local_seconds)
    return total / slowest, total, slowest
