"""GPU exact k-NN (BruteForceIndex) against the reference's brute-force results."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _eq(rec, want_l, want_d, what):
    np.testing.assert_array_equal(rec["label"].astype(np.int64), want_l, err_msg=what)
    assert rec["distance"].tobytes() == want_d.astype(np.float32).tobytes(), what


def test_l2_integer_data(hg, golden, graphs):
    _, arr = golden
    base, q, *_ = graphs.data("c1")
    bf = hg.BruteForceIndex(128, "l2")
    bf.add(base)
    _eq(bf.search_raw(q[:200], 10), arr["c1_bf_labels"], arr["c1_bf_dists"], "c1")


def test_cosine_with_filter_masked_tail(hg, golden, graphs):
    _, arr = golden
    import workloads

    base, q, *_ = graphs.data("c3s")  # d = 100: 64-block, two 16-blocks, a 4-float masked tail
    bf = hg.BruteForceIndex(100, "cosine")
    bf.add(base)
    fw = workloads.label_filter_bits(4000, lambda x: x % 10 == 0)
    _eq(bf.search_raw(q[:100], 10, filter=hg.Bitset(fw, 4000)), arr["c3s_bf_f_labels"], arr["c3s_bf_f_dists"], "c3s")


def test_high_dim(hg, golden, graphs):
    _, arr = golden
    base, q, *_ = graphs.data("c4s")
    bf = hg.BruteForceIndex(960, "l2")
    bf.add(base)
    _eq(bf.search_raw(q[:50], 10), arr["c4s_bf_labels"], arr["c4s_bf_dists"], "c4s")


def test_edge_cases(hg, oracle):
    rng = np.random.default_rng(4)
    data = rng.uniform(-1, 1, size=(3, 4)).astype(np.float32)
    bf = hg.BruteForceIndex(4, "ip")
    bf.add(data)
    rec = bf.search_raw(data[:1], 10)  # k > size: padded
    assert (rec["label"][0, 3:] == hg.INVALID_LABEL).all()
    ol, od = oracle.bruteforce(data, data[:1], 10, "ip")
    np.testing.assert_array_equal(rec["label"], ol)
    # labels not in insertion order: ties broken by label
    lab = np.array([50, 7, 30], dtype=np.uint64)
    same = np.ones((3, 4), dtype=np.float32)
    bf2 = hg.BruteForceIndex(4, "l2")
    bf2.add(same, lab)
    rec = bf2.search_raw(same[:1], 3)
    assert list(rec["label"][0]) == [7, 30, 50]
    with pytest.raises(ValueError):
        bf2.search_raw(same[:1], 0)
