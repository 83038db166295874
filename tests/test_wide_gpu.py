"""Several warps per query (warps_per_query=4) for the compressed forms.

Layer 0 is a beam search expanding four candidates per step, so the visit
order is not the reference's and results are held to a recall bar: every
returned distance must still be the exact FP32 distance of that id
(bitwise), rows sorted by (distance, label), and the overlap with the exact
path close to the one-warp compressed form's.
"""
from __future__ import annotations

import numpy as np
import pytest

from test_precision_gpu import _check

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [1, 2])
def test_wide_distances_exact_and_recall(hg, oracle, graphs, prec):
    base, q, *_ = graphs.data("c1")
    ix = hg.Index.load(graphs.path("c1"))
    o_one = _check(hg, oracle, ix, base, q[:200], 10, 80, prec, "l2", 0.85)
    o_wide = _check(hg, oracle, ix, base, q[:200], 10, 80, prec, "l2", 0.85, warps_per_query=4)
    assert o_wide >= o_one - 0.03, (o_wide, o_one)


def test_wide_mixed_batch_pads_and_matches_alone(hg, graphs):
    _, q, *_ = graphs.data("c1")
    ix = hg.Index.load(graphs.path("c1"))
    rng = np.random.default_rng(3)
    efs = rng.choice([16, 40, 100, 300], q.shape[0]).astype(np.uint32)
    ks = rng.choice([1, 5, 10], q.shape[0]).astype(np.uint32)
    rec = ix.search_batch_ex(q, 10, ef_per_query=efs, k_per_query=ks, precision=2, warps_per_query=4)
    for i in range(0, q.shape[0], 37):
        k = int(ks[i])
        assert (rec["label"][i, k:] == np.uint64(~np.uint64(0))).all()
        assert np.isinf(rec["distance"][i, k:]).all()
        alone = ix.search_batch_ex(q[i:i + 1], k, int(efs[i]), precision=2, warps_per_query=4)
        np.testing.assert_array_equal(alone["label"][0], rec["label"][i, :k])
        assert alone["distance"][0].tobytes() == rec["distance"][i, :k].tobytes()


@pytest.mark.parametrize("prec", [1, 2])
def test_wide_cosine_filters_deletes(hg, graphs, prec):
    import workloads

    _, q, *_ = graphs.data("c3s")  # d = 100 -> rows padded to 128
    ix = hg.Index.load(graphs.path("c3s", deleted=True))
    fw = workloads.label_filter_bits(4000, lambda l: l % 2 == 0)
    rec = ix.search_batch_ex(q, 10, 160, precision=prec, filters=[hg.Bitset(fw, 4000)], warps_per_query=4)
    labels = rec["label"].astype(np.int64)
    deleted = set(workloads.random_deletes(4000, 0.01, seed=2).tolist())
    for row in labels:
        for l in row:
            assert l == -1 or (l % 2 == 0 and l not in deleted)
    exact = ix.search_raw(q, 10, 160, filter=hg.Bitset(fw, 4000))
    overlap = np.mean([len(set(a) & set(b)) / 10 for a, b in zip(labels, exact["label"].astype(np.int64))])
    assert overlap >= 0.85, overlap


def test_wide_server_same_result_alone_and_in_the_mix(hg, graphs):
    _, q, *_ = graphs.data("c1")
    ix = hg.Index.load(graphs.path("c1"))
    srv = hg.Server(ix, precision=2, warps_per_query=4, rerank_factor=4, max_batch_queries=256)
    rng = np.random.default_rng(5)
    reqs = []
    for i in range(60):
        n = int(rng.integers(1, 20))
        s = int(rng.integers(0, q.shape[0] - n))
        reqs.append((q[s:s + n], int(rng.choice([1, 10])), int(rng.choice([20, 100, 200])), None))
    _, outs = srv.replay(reqs, np.zeros(len(reqs)))
    for (qq, k, ef, _), out in zip(reqs, outs):
        alone = ix.search_batch_ex(qq, k, ef, precision=2, warps_per_query=4, rerank_factor=4)
        np.testing.assert_array_equal(out["label"], alone["label"])
        assert out["distance"].tobytes() == alone["distance"].tobytes()
    srv.close()
