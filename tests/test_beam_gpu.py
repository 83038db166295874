"""The beam walk of the compressed-precision forms (lists_per_step = 1..4):
one warp per query, several neighbour lists per step, row distances on the
tensor cores, then the exact FP32 rerank.

Its visit order is not the reference's, so the bar is the precision form's:
every returned distance equals the exact FP32 distance of its id (bitwise),
rows are sorted by (distance, label), filters and deletes are honoured, and
the answers overlap the exact path's.  Each answer depends on its query
alone, so it is the same in any batch.
"""
from __future__ import annotations

import numpy as np
import pytest

from test_precision_gpu import _check

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("lists", [1, 2, 4])
@pytest.mark.parametrize("prec,min_overlap", [(1, 0.97), (2, 0.85)])
def test_integer_l2(hg, oracle, graphs, prec, min_overlap, lists):
    base, q, *_ = graphs.data("c1")
    ix = hg.Index.load(graphs.path("c1"))
    for ef in (40, 160):
        _check(hg, oracle, ix, base, q[:200], 10, ef, prec, "l2", min_overlap, lists_per_step=lists)


@pytest.mark.parametrize("prec", [1, 2])
def test_inner_product(hg, oracle, graphs, prec):
    base, q, *_ = graphs.data("ip")
    ix = hg.Index.load(graphs.path("ip"))
    _check(hg, oracle, ix, base, q[:100], 10, 80, prec, "ip", 0.85, lists_per_step=2)


@pytest.mark.parametrize("prec", [1, 2])
def test_cosine_filters_deletes(hg, oracle, graphs, prec):
    import workloads

    base, q, *_ = graphs.data("c3s")  # d = 100 -> rows padded to 128
    ix = hg.Index.load(graphs.path("c3s", deleted=True))
    fw = workloads.label_filter_bits(4000, lambda l: l % 2 == 0)
    rec = ix.search_batch_ex(q, 10, 160, precision=prec, filters=[hg.Bitset(fw, 4000)], lists_per_step=4)
    labels = rec["label"].astype(np.int64)
    deleted = set(workloads.random_deletes(4000, 0.01, seed=2).tolist())
    for row in labels:
        for lab in row:
            assert lab == -1 or (lab % 2 == 0 and lab not in deleted)
    exact = ix.search_raw(q, 10, 160, filter=hg.Bitset(fw, 4000))
    overlap = np.mean([len(set(a) & set(b)) / 10 for a, b in zip(labels, exact["label"].astype(np.int64))])
    assert overlap >= 0.9, overlap
    # unfiltered queries on the index with deletes never return a deleted label
    rec = ix.search_batch_ex(q, 10, 80, precision=prec, lists_per_step=2)
    assert not (set(rec["label"].astype(np.int64).ravel().tolist()) & deleted)


def test_forgetful_visited_set(hg, oracle, graphs):
    """Large ef fills the small visited hash, which restarts holding the beam
    (counter 7 counts the restarts): answers keep the exact distances, no
    duplicate labels, and the quality of the exact path."""
    base, q, *_ = graphs.data("c1")
    ix = hg.Index.load(graphs.path("c1"))
    _, cnt = ix.search_batch_ex(q[:100], 10, 400, precision=1, lists_per_step=4, counters=True)
    assert (cnt[:, 7] > 0).sum() > 50, cnt[:, 7]
    _check(hg, oracle, ix, base, q[:100], 10, 400, 1, "l2", 0.97, lists_per_step=4)


def test_answers_do_not_depend_on_the_batch(hg, graphs):
    _, q, *_ = graphs.data("c1")
    ix = hg.Index.load(graphs.path("c1"))
    efs = np.random.default_rng(5).choice(np.array([16, 40, 100, 300], np.uint32), q.shape[0])
    ks = np.random.default_rng(6).choice(np.array([1, 10, 50], np.uint32), q.shape[0])
    mixed = ix.search_batch_ex(q, 50, ef_per_query=efs, k_per_query=ks, precision=2, lists_per_step=4,
                               rerank_factor=4)
    for i in range(0, q.shape[0], 97):
        alone = ix.search_batch_ex(q[i:i + 1], int(ks[i]), int(efs[i]), precision=2, lists_per_step=4,
                                   rerank_factor=4)
        assert alone.tobytes() == mixed[i:i + 1, :int(ks[i])].tobytes(), i


def test_recall_close_to_exact_path(hg, graphs):
    """Recall@10 against exact k-NN (integer data: FP32 brute force is exact)."""
    import workloads

    base, q, *_ = graphs.data("c1")
    ix = hg.Index.load(graphs.path("c1"))
    bf = hg.BruteForceIndex(base.shape[1], "l2")
    bf.add(base)
    gt = bf.search_raw(q, 10)["label"].astype(np.int64)
    exact = workloads.recall_at_k(ix.search_raw(q, 10, 40)["label"].astype(np.int64), gt)
    for prec in (1, 2):
        for lists in (1, 4):
            got = ix.search_batch_ex(q, 10, 40, precision=prec, lists_per_step=lists, rerank_factor=4)
            r = workloads.recall_at_k(got["label"].astype(np.int64), gt)
            assert r >= exact - (0.01 if prec == 1 else 0.03), (prec, lists, r, exact)
