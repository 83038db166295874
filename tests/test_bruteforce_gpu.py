"""GPU exact k-NN (BruteForceIndex) against the reference's brute-force results.

Both kernels are held to the same bar: the CUDA-core scan and the
tensor-core path (FP16 tcgen05 GEMM, margin selection, exact rerank in the
reference order) must give ids and distances bit-identical to the
reference's, and the tensor path must be the one that answered.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _eq(rec, want_l, want_d, what):
    np.testing.assert_array_equal(rec["label"].astype(np.int64), want_l, err_msg=what)
    assert rec["distance"].tobytes() == want_d.astype(np.float32).tobytes(), what


PATHS = [1, 2]  # CUDA-core scan, tensor cores


def _bf(hg, dim, metric, base, path, labels=None):
    bf = hg.BruteForceIndex(dim, metric)
    bf.add(base, labels)
    bf.set_path(path)
    return bf


def _answered(bf, path):
    assert bf.last_path == path, f"path {path} requested, {bf.last_path} answered"


@pytest.mark.parametrize("path", PATHS)
def test_l2_integer_data(hg, golden, graphs, path):
    _, arr = golden
    base, q, *_ = graphs.data("c1")
    bf = _bf(hg, 128, "l2", base, path)
    _eq(bf.search_raw(q[:200], 10), arr["c1_bf_labels"], arr["c1_bf_dists"], "c1")
    _answered(bf, path)


@pytest.mark.parametrize("path", PATHS)
def test_cosine_with_filter_masked_tail(hg, golden, graphs, path):
    _, arr = golden
    import workloads

    base, q, *_ = graphs.data("c3s")  # d = 100: 64-block, two 16-blocks, a 4-float masked tail
    bf = _bf(hg, 100, "cosine", base, path)
    fw = workloads.label_filter_bits(4000, lambda x: x % 10 == 0)
    _eq(bf.search_raw(q[:100], 10, filter=hg.Bitset(fw, 4000)), arr["c3s_bf_f_labels"], arr["c3s_bf_f_dists"], "c3s")
    _answered(bf, path)


@pytest.mark.parametrize("path", PATHS)
def test_high_dim(hg, golden, graphs, path):
    _, arr = golden
    base, q, *_ = graphs.data("c4s")
    bf = _bf(hg, 960, "l2", base, path)
    _eq(bf.search_raw(q[:50], 10), arr["c4s_bf_labels"], arr["c4s_bf_dists"], "c4s")
    _answered(bf, path)


@pytest.mark.parametrize("path", PATHS)
def test_edge_cases(hg, oracle, path):
    rng = np.random.default_rng(4)
    data = rng.uniform(-1, 1, size=(3, 4)).astype(np.float32)
    bf = _bf(hg, 4, "ip", data, path)
    rec = bf.search_raw(data[:1], 10)  # k > size: padded
    assert (rec["label"][0, 3:] == hg.INVALID_LABEL).all()
    ol, od = oracle.bruteforce(data, data[:1], 10, "ip")
    np.testing.assert_array_equal(rec["label"], ol)
    # labels not in insertion order: ties broken by label
    lab = np.array([50, 7, 30], dtype=np.uint64)
    same = np.ones((3, 4), dtype=np.float32)
    bf2 = _bf(hg, 4, "l2", same, path, lab)
    rec = bf2.search_raw(same[:1], 3)
    assert list(rec["label"][0]) == [7, 30, 50]
    with pytest.raises(ValueError):
        bf2.search_raw(same[:1], 0)


@pytest.mark.parametrize("metric", ["l2", "ip", "cosine"])
def test_tensor_path_float_data_vs_oracle(hg, oracle, metric):
    """Gaussian float data (the margin path): several k, a filter, a query
    count that spans many base splits and one that fills many tiles."""
    import workloads

    rng = np.random.default_rng(11)
    base = rng.normal(size=(20_000, 72)).astype(np.float32)
    q = rng.normal(size=(300, 72)).astype(np.float32)
    bf = _bf(hg, 72, metric, base, 2)
    for k in (1, 10, 100, 256):
        rec = bf.search_raw(q[:40], k)
        ol, od = oracle.bruteforce(base, q[:40], k, metric)
        _eq(rec, ol.astype(np.int64), od, f"{metric} k={k}")
        _answered(bf, 2)
    fw = workloads.label_filter_bits(20_000, lambda x: x % 7 == 3)
    rec = bf.search_raw(q, 10, filter=hg.Bitset(fw, 20_000))
    ol, od = oracle.bruteforce(base, q, 10, metric, filt=(fw, 20_000))
    _eq(rec, ol.astype(np.int64), od, f"{metric} filtered")
    _answered(bf, 2)


def test_tensor_path_many_queries_and_ties(hg, oracle):
    """20,000 queries (more query tiles than SMs) on integer data with many
    duplicate rows: exact mode (zero margin) with ties broken by label."""
    rng = np.random.default_rng(12)
    base = rng.integers(0, 8, size=(6000, 16)).astype(np.float32)  # many equal rows and distances
    q = rng.integers(0, 8, size=(20_000, 16)).astype(np.float32)
    labels = rng.permutation(6000).astype(np.uint64) * 3
    bf = _bf(hg, 16, "l2", base, 2, labels)
    rec = bf.search_raw(q, 5)
    ol, od = oracle.bruteforce(base, q, 5, "l2", labels=labels)
    _eq(rec, ol.astype(np.int64), od, "ties")
    scan = _bf(hg, 16, "l2", base, 1, labels)
    np.testing.assert_array_equal(scan.search_raw(q[:500], 5)["label"], rec[:500]["label"])


def test_auto_path_uses_tensor_cores(hg, graphs):
    base, q, *_ = graphs.data("c1")
    bf = hg.BruteForceIndex(128, "l2")
    bf.add(base)
    bf.search_raw(q[:10], 10)
    assert bf.last_path == 2


def test_seeded_thresholds_large_k(hg, oracle):
    """k >= 64 over >= 2,048 queries: the GEMM first runs a bound pass that
    keeps each (query, half tile)'s smallest score, and every query's scan
    starts from the k-th smallest of those minima plus its margin.  Float
    data (margin path) with and without a filter, and integer data with many
    ties (exact mode), against the oracle."""
    import workloads

    rng = np.random.default_rng(13)
    base = rng.normal(size=(30_000, 48)).astype(np.float32)
    q = rng.normal(size=(2_100, 48)).astype(np.float32)
    bf = _bf(hg, 48, "l2", base, 2)
    rec = bf.search_raw(q, 100)
    ol, od = oracle.bruteforce(base, q, 100, "l2")
    _eq(rec, ol.astype(np.int64), od, "seeded k=100")
    _answered(bf, 2)
    fw = workloads.label_filter_bits(30_000, lambda x: x % 5 == 1)
    rec = bf.search_raw(q, 64, filter=hg.Bitset(fw, 30_000))
    ol, od = oracle.bruteforce(base, q, 64, "l2", filt=(fw, 30_000))
    _eq(rec, ol.astype(np.int64), od, "seeded k=64 filtered")
    ints = rng.integers(0, 8, size=(6000, 16)).astype(np.float32)
    qi = rng.integers(0, 8, size=(2_500, 16)).astype(np.float32)
    bi = _bf(hg, 16, "l2", ints, 2)
    rec = bi.search_raw(qi, 80)
    ol, od = oracle.bruteforce(ints, qi, 80, "l2")
    _eq(rec, ol.astype(np.int64), od, "seeded ties")
