"""Query sharding across GPU replicas.

Queries are independent and every GPU holds the whole graph, so N GPUs serve
a batch as N replicas: rank r answers the contiguous slice shard_bounds(nq, r, N)
of the queries on its own GPU, and the rows are concatenated in rank order.
There is no collective on the data path; the only exchanges are the result
gather (one all_gather of the records' bytes) and the timing reduction (max
over ranks).  A partition of the graph itself would change the answers, so
it is not offered.
"""
from __future__ import annotations

import numpy as np


def shard_bounds(nq: int, rank: int, world: int) -> tuple[int, int]:
    """[lo, hi) of rank's queries: contiguous, sizes differ by at most one."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("shard_bounds: need 0 <= rank < world")
    return nq * rank // world, nq * (rank + 1) // world


RECORD = np.dtype([("label", "<u8"), ("distance", "<f4"), ("reserved", "<u4")])  # hnsw::Neighbor


def search_sharded(index, queries, k: int, rank: int, world: int, group=None, **search_kw) -> np.ndarray:
    """Answer this rank's slice of `queries` with index.search_batch_ex and
    gather every rank's rows into the full nq x k record array, identical on
    every rank.  The gather moves the records as raw bytes in one tensor
    all_gather (device tensors under NCCL, host tensors otherwise), each
    rank's slice padded to the largest slice's rows (slices differ by at
    most one row)."""
    import torch
    import torch.distributed as dist

    q = np.ascontiguousarray(queries, dtype=np.float32)
    nq = q.shape[0]
    lo, hi = shard_bounds(nq, rank, world)
    kw = dict(search_kw)
    for name in ("ef_per_query", "k_per_query", "filter_of_query"):
        if kw.get(name) is not None:
            kw[name] = np.asarray(kw[name])[lo:hi]
    rows_max = -(-nq // world)
    row_bytes = k * RECORD.itemsize
    buf = np.zeros(rows_max * row_bytes, dtype=np.uint8)
    if hi > lo:
        local = np.ascontiguousarray(index.search_batch_ex(q[lo:hi], k, **kw)).reshape(-1)
        buf[: local.nbytes] = local.view(np.uint8)
    on_gpu = dist.get_backend(group) == "nccl"
    dev = torch.device("cuda", torch.cuda.current_device()) if on_gpu else torch.device("cpu")
    mine = torch.from_numpy(buf).to(dev)
    parts = [torch.empty_like(mine) for _ in range(world)]
    dist.all_gather(parts, mine, group=group)
    out = np.empty((nq, k), dtype=RECORD)
    flat = out.reshape(-1).view(np.uint8)
    for r, t in enumerate(parts):
        a, b = shard_bounds(nq, r, world)
        flat[a * row_bytes: b * row_bytes] = t.cpu().numpy()[: (b - a) * row_bytes]
    return out


def max_over_ranks(value: float, group=None) -> float:
    """The job's time for a step: the slowest rank's."""
    import torch
    import torch.distributed as dist

    on_gpu = dist.get_backend(group) == "nccl"  # NCCL reduces device tensors only
    dev = torch.device("cuda", torch.cuda.current_device()) if on_gpu else torch.device("cpu")
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())
