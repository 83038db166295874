"""Replica sharding (multi-GPU path) on CPU: world_size-2 gloo process groups.

The GPU search is replaced by the oracle's CPU search over the same graph
file (the checker), so what is tested is the host logic the N-GPU path adds:
the query split, the per-rank ef / k slices, the gather in rank order and the
max-over-ranks timing reduction.
"""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest

from conftest import GOLD


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


class _OracleIndex:
    """search_batch_ex over the oracle (per-query ef / k), the GPU stand-in."""

    def __init__(self, path):
        import pyoracle

        self.ox = pyoracle.OracleIndex(path)

    def search_batch_ex(self, q, k, ef_per_query=None, k_per_query=None):
        labels, dists = self.ox.search_batch(q, k, 0, ef_per_query=ef_per_query, k_per_query=k_per_query)
        rec = np.zeros(labels.shape, dtype=[("label", "<u8"), ("distance", "<f4"), ("reserved", "<u4")])
        rec["label"], rec["distance"] = labels, dists
        return rec


def _worker(rank, world, port, path, q, efs, ks, out_dir):
    import sys

    import torch.distributed as dist

    sys.path[:0] = [os.path.join(os.path.dirname(__file__), "..", "hnsw-engine_gb300"),
                    os.path.join(os.path.dirname(__file__), "..", "oracle")]
    import replicas

    os.environ["MASTER_ADDR"], os.environ["MASTER_PORT"] = "127.0.0.1", str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        rows = replicas.search_sharded(_OracleIndex(path), q, 10, rank, world, ef_per_query=efs, k_per_query=ks)
        t = replicas.max_over_ranks(1.0 + rank)
        np.save(os.path.join(out_dir, f"rows{rank}.npy"), rows)
        np.save(os.path.join(out_dir, f"t{rank}.npy"), np.array([t]))
    finally:
        dist.destroy_process_group()


def test_shard_bounds_cover_every_query_once():
    import replicas

    for nq in (0, 1, 7, 10_000):
        for world in (1, 2, 3, 8):
            seen = []
            for r in range(world):
                lo, hi = replicas.shard_bounds(nq, r, world)
                seen.extend(range(lo, hi))
                assert hi - lo in (nq // world, nq // world + 1)
            assert seen == list(range(nq))
    with pytest.raises(ValueError):
        replicas.shard_bounds(10, 2, 2)


@pytest.mark.parametrize("world", [2])
def test_two_replicas_equal_one(tmp_path, world):
    import torch.multiprocessing as mp

    path = GOLD / "persist.idx"
    import pyoracle

    ox = pyoracle.OracleIndex(path)
    dim = ox.dim
    rng = np.random.default_rng(3)
    q = rng.normal(size=(37, dim)).astype(np.float32)
    efs = rng.choice(np.array([10, 20, 40], dtype=np.uint64), q.shape[0])
    ks = rng.choice(np.array([1, 5, 10], dtype=np.uint64), q.shape[0])
    want = _OracleIndex(path).search_batch_ex(q, 10, ef_per_query=efs, k_per_query=ks)
    mp.start_processes(_worker, args=(world, _free_port(), str(path), q, efs, ks, str(tmp_path)), nprocs=world,
                       join=True, start_method="spawn")
    for r in range(world):
        got = np.load(tmp_path / f"rows{r}.npy")
        np.testing.assert_array_equal(got["label"], want["label"])
        assert got["distance"].tobytes() == want["distance"].tobytes()
        assert float(np.load(tmp_path / f"t{r}.npy")[0]) == float(world)
