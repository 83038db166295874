"""Parity at the stated sizes of the cosine-with-filters workload and the
d = 960 workload.

* cosine, filters and deletes: n = 200,000, d = 100 unit vectors (1,000
  random unit centres plus N(0, 0.3^2) noise, renormalised), 10,000
  queries; M = 16, ef_construction = 200; 1% of the labels soft-deleted
  (seed 2); half of the queries filtered to labels with label % 10 == 0;
  k in {10, 100}, ef in {40, 100, 200, 400} per query.  The GPU answers all
  10,000 queries in one batch (per-query k, ef and filter); the checker
  answers one call per (filtered, k, ef) group, as the reference's API
  takes one k / ef / filter per call.
* d = 960: n = 200,000 rows of |N(0, 1)| times per-dimension scales from
  U[0.05, 1], 5,000 queries, k = 10, ef in {40, 128, 512}.

The checker is the reference's own search_batch (compiled from its sources
on this host) on the graph its own add_batch built, in the summation order
of this host's reference kernels; where the reference is not built, the
oracle (its C restatement) in the AVX-512 order.  Ids and distance bits must
be equal for every query.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 200_000


def _checker(hg, tmp_path, base, metric, tag):
    """(order, path, kind): the graph file and the order both sides use."""
    import refcore

    if refcore.available() and refcore.isa() in ("neon", "avx512"):
        path = refcore.build(base, tmp_path / f"{tag}.idx", metric=metric, M=16, ef_construction=200, threads=0)
        return refcore.isa(), path, "reference"
    ix = hg.Index(base.shape[1], metric, 16, 200)
    ix.add(base)  # all host threads: the graph is only the input here
    path = tmp_path / f"{tag}.idx"
    ix.save(path)
    return "avx512", path, "oracle"


def _assert_rows_equal(gpu_rows, labels, dists, what):
    bad = np.nonzero((gpu_rows["label"] != labels).any(1) |
                     (gpu_rows["distance"].view(np.uint32) != dists.view(np.uint32)).any(1))[0]
    assert bad.size == 0, f"{what}: {bad.size} queries differ, first {bad[:5].tolist()}"


def test_cosine_filters_deletes_at_size(hg, oracle, tmp_path):
    import workloads

    base, q = workloads.unit_mixture(N, 100, 1000, 10_000)
    order, path, kind = _checker(hg, tmp_path, base, "cosine", "cos200k")
    dels = workloads.random_deletes(N, 0.01, seed=2)
    fw = workloads.label_filter_bits(N, lambda l: l % 10 == 0)
    rng = np.random.default_rng(3)
    filt = rng.random(q.shape[0]) < 0.5
    ks = rng.choice([10, 100], size=q.shape[0]).astype(np.uint32)
    efs = rng.choice([40, 100, 200, 400], size=q.shape[0]).astype(np.uint32)

    hg.set_distance_order(order)
    try:
        ix = hg.Index.load(path)
    finally:
        hg.set_distance_order("avx512")
    for lab in dels:
        ix.mark_deleted(int(lab))
    rec = ix.search_batch_ex(q, 100, ef_per_query=efs, k_per_query=ks, filters=[hg.Bitset(fw, N)],
                             filter_of_query=np.where(filt, 0, -1).astype(np.int32))

    if kind == "reference":
        import refcore

        rx = refcore.RefIndex(path)
        for lab in dels:
            rx.mark_deleted(int(lab))
        bits = refcore.Bitset(fw, N)
    else:
        ox = oracle.OracleIndex(path, isa=order)
        for lab in dels:
            ox.mark_deleted(int(lab))
    groups = 0
    for f in (False, True):
        for k in (10, 100):
            for ef in (40, 100, 200, 400):
                sel = np.nonzero((filt == f) & (ks == k) & (efs == ef))[0]
                if sel.size == 0:
                    continue
                groups += 1
                if kind == "reference":
                    r = rx.search_batch(q[sel], k, ef, threads=0, filt=bits if f else None)
                    labels, dists = r["label"], r["distance"]
                else:
                    labels, dists = ox.search_batch(q[sel], k, ef, filters=[(fw, N)] if f else None,
                                                    fsel=np.zeros(sel.size, np.int32) if f else None)
                _assert_rows_equal(rec[sel, :k], labels, dists, f"{kind} k={k} ef={ef} filtered={f}")
                assert (rec[sel, k:]["label"] == hg.INVALID_LABEL).all()
    assert groups == 16


def test_d960_at_size(hg, oracle, tmp_path):
    import workloads

    base, q = workloads.scaled_abs_normal(N, 960, 5_000)
    order, path, kind = _checker(hg, tmp_path, base, "l2", "d960")
    hg.set_distance_order(order)
    try:
        ix = hg.Index.load(path)
    finally:
        hg.set_distance_order("avx512")
    if kind == "reference":
        import refcore

        rx = refcore.RefIndex(path)
    else:
        ox = oracle.OracleIndex(path, isa=order)
    for ef in (40, 128, 512):
        rec = ix.search_raw(q, 10, ef)
        if kind == "reference":
            r = rx.search_batch(q, 10, ef, threads=0)
            labels, dists = r["label"], r["distance"]
        else:
            labels, dists = ox.search_batch(q, 10, ef)
        _assert_rows_equal(rec, labels, dists, f"{kind} d=960 ef={ef}")
