"""Query sharding across GPU replicas.

Queries are independent and every GPU holds the whole graph, so N GPUs serve
a batch as N replicas: rank r answers the contiguous slice shard_bounds(nq, r, N)
of the queries on its own GPU, and the rows are concatenated in rank order.
There is no collective on the data path; the only exchanges are the result
gather (host side) and the timing reduction (max over ranks).  A partition of
the graph itself would change the answers, so it is not offered.
"""
from __future__ import annotations

import numpy as np


def shard_bounds(nq: int, rank: int, world: int) -> tuple[int, int]:
    """[lo, hi) of rank's queries: contiguous, sizes differ by at most one."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("shard_bounds: need 0 <= rank < world")
    return nq * rank // world, nq * (rank + 1) // world


def search_sharded(index, queries, k: int, rank: int, world: int, group=None, **search_kw) -> np.ndarray:
    """Answer this rank's slice of `queries` with index.search_batch_ex and
    gather every rank's rows (torch.distributed, any backend) into the full
    nq x k record array, identical on every rank."""
    import torch.distributed as dist

    q = np.ascontiguousarray(queries, dtype=np.float32)
    lo, hi = shard_bounds(q.shape[0], rank, world)
    kw = dict(search_kw)
    for name in ("ef_per_query", "k_per_query", "filter_of_query"):
        if kw.get(name) is not None:
            kw[name] = np.asarray(kw[name])[lo:hi]
    local = index.search_batch_ex(q[lo:hi], k, **kw) if hi > lo else None
    parts = [None] * world
    dist.all_gather_object(parts, local, group=group)
    rows = [p for p in parts if p is not None]
    return np.concatenate(rows, axis=0) if rows else np.empty((0, k), dtype=np.dtype([("label", "<u8"),
                                                                                     ("distance", "<f4"),
                                                                                     ("pad", "<u4")]))


def max_over_ranks(value: float, group=None) -> float:
    """The job's time for a step: the slowest rank's."""
    import torch
    import torch.distributed as dist

    on_gpu = dist.get_backend(group) == "nccl"  # NCCL reduces device tensors only
    dev = torch.device("cuda", torch.cuda.current_device()) if on_gpu else torch.device("cpu")
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())
