"""FP16 / FP8-E4M3 traversal with an exact FP32 rerank.

The traversal walks the same graph with the same visited set and filters,
but computes distances on compressed rows; the final pool is reranked with
exact FP32 distances in the reference's order.  So every returned distance
must equal the exact distance of that id (bitwise), rows must be sorted by
(distance, label), and recall must stay close to the exact path's.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _check(hg, oracle, ix, base, q, k, ef, prec, metric, min_overlap, rerank_factor=0, **kw):
    exact = ix.search_raw(q, k, ef)
    rec = ix.search_batch_ex(q, k, ef, precision=prec, rerank_factor=rerank_factor, **kw)
    labels = rec["label"].astype(np.int64)
    assert (labels >= 0).all()
    for i in range(q.shape[0]):
        assert len(set(labels[i].tolist())) == k
        pq = oracle.prepare_vector(metric, q[i])
        for j in range(k):
            v = oracle.prepare_vector(metric, base[labels[i, j]])
            pdim = -(-base.shape[1] // 16) * 16
            a = np.zeros(pdim, np.float32)
            b = np.zeros(pdim, np.float32)
            a[:base.shape[1]], b[:base.shape[1]] = pq, v
            want = oracle.lib().orc_distance(oracle.ISAS["avx512"], oracle.METRICS[metric],
                                             a.ctypes.data, b.ctypes.data, pdim)
            assert np.float32(want).tobytes() == rec["distance"][i, j].tobytes(), (i, j)
        d = rec["distance"][i]
        assert all((d[t], labels[i, t]) <= (d[t + 1], labels[i, t + 1]) for t in range(k - 1))
    overlap = np.mean([len(set(a) & set(b)) / k for a, b in zip(labels, exact["label"].astype(np.int64))])
    assert overlap >= min_overlap, (prec, overlap)
    return overlap


@pytest.mark.parametrize("prec,min_overlap", [(1, 0.97), (2, 0.85)])
def test_integer_l2(hg, oracle, graphs, prec, min_overlap):
    base, q, *_ = graphs.data("c1")
    ix = hg.Index.load(graphs.path("c1"))
    _check(hg, oracle, ix, base, q[:200], 10, 80, prec, "l2", min_overlap)


@pytest.mark.parametrize("prec,min_overlap", [(1, 0.97), (2, 0.85)])
def test_float_highdim(hg, oracle, graphs, prec, min_overlap):
    base, q, *_ = graphs.data("c4s")  # d = 960 -> rows padded to 1024
    ix = hg.Index.load(graphs.path("c4s"))
    _check(hg, oracle, ix, base, q[:50], 10, 80, prec, "l2", min_overlap)


@pytest.mark.parametrize("prec", [1, 2])
def test_cosine_filters_deletes(hg, oracle, graphs, prec):
    import workloads

    base, q, *_ = graphs.data("c3s")  # d = 100 -> rows padded to 128
    ix = hg.Index.load(graphs.path("c3s", deleted=True))
    fw = workloads.label_filter_bits(4000, lambda l: l % 10 == 0)
    rec = ix.search_batch_ex(q, 10, 160, precision=prec, filters=[hg.Bitset(fw, 4000)])
    labels = rec["label"].astype(np.int64)
    deleted = set(workloads.random_deletes(4000, 0.01, seed=2).tolist())
    for row in labels:
        for l in row:
            assert l == -1 or (l % 10 == 0 and l not in deleted)
    exact = ix.search_raw(q, 10, 160, filter=hg.Bitset(fw, 4000))
    overlap = np.mean([len(set(a) & set(b)) / 10 for a, b in zip(labels, exact["label"].astype(np.int64))])
    assert overlap >= 0.9


@pytest.mark.parametrize("prec", [1, 2])
def test_rerank_factor(hg, oracle, graphs, prec):
    """A rerank factor covering the whole pool changes nothing; a small one
    reranks only the pool's best factor x k, with distances still exact."""
    base, q, *_ = graphs.data("c1")
    ix = hg.Index.load(graphs.path("c1"))
    full = ix.search_batch_ex(q[:200], 10, 200, precision=prec)
    covering = ix.search_batch_ex(q[:200], 10, 200, precision=prec, rerank_factor=20)  # 20 x 10 >= ef
    assert full.tobytes() == covering.tobytes()
    o_full = _check(hg, oracle, ix, base, q[:200], 10, 200, prec, "l2", 0.85)
    o_part = _check(hg, oracle, ix, base, q[:200], 10, 200, prec, "l2", 0.85, rerank_factor=4)
    assert o_part >= o_full - 0.01, (o_part, o_full)
