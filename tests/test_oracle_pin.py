"""Pin the oracle (the C restatement under oracle/) to the reference itself.

Every expectation here is an output of the reference hnsw-engine, produced by
tests/golden/make_golden.py: raw distance kernels per ISA, search_batch /
search results on graphs the reference built and saved, brute-force results,
and the corrupted files its loader rejects.  CPU only.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import GOLD, sha256


def test_kernels_bitwise_per_isa(oracle, golden):
    meta, arr = golden
    kin = np.load(GOLD / "kernel_inputs.npz")
    for isa in meta["kernels"]["isas"]:
        for d in meta["kernels"]["dims"]:
            want = arr[f"kern_{isa}_{d}"]
            a, b = kin[f"a{d}"], kin[f"b{d}"]
            for i in range(a.shape[0]):
                l2 = oracle.kernel(isa, True, a[i], b[i])
                dp = oracle.kernel(isa, False, a[i], b[i])
                assert l2.tobytes() == want[i, 0].tobytes(), (isa, d, i)
                assert dp.tobytes() == want[i, 1].tobytes(), (isa, d, i)


def test_exact_small_integer_kernels(oracle):
    # test_kernels.cpp:44-58: small-integer vectors give exact sums in every order
    for d in [1, 7, 8, 9, 15, 16, 17, 31, 33, 63, 64, 65, 100, 128, 960]:
        a = (np.arange(d) % 7 - 3).astype(np.float32)
        b = (np.arange(d) % 5 - 2).astype(np.float32)
        l2 = float(((a.astype(np.float64) - b) ** 2).sum())
        dp = float((a.astype(np.float64) * b).sum())
        for isa in ("scalar", "avx2", "avx512", "neon"):
            assert oracle.kernel(isa, True, a, b) == np.float32(l2)
            assert oracle.kernel(isa, False, a, b) == np.float32(dp)


def _same(got_l, got_d, want_l, want_d):
    gl = got_l.astype(np.int64)
    np.testing.assert_array_equal(gl, want_l)
    assert got_d.tobytes() == want_d.astype(np.float32).tobytes()


def test_small_reference_files(oracle, golden):
    meta, arr = golden
    for name, h in meta["small"].items():
        assert sha256(GOLD / f"{name}.idx") == h
    ix = oracle.OracleIndex(GOLD / "dim1.idx")
    l, d = ix.search(np.array([42.2], dtype=np.float32), 3, 50)
    _same(l, d, arr["dim1_labels"], arr["dim1_dists"])
    assert list(l) == [42, 43, 41]
    ix = oracle.OracleIndex(GOLD / "identical.idx")
    l, d = ix.search(np.full(12, 0.5, dtype=np.float32), 10, 64)
    _same(l, d, arr["identical_labels"], arr["identical_dists"])
    assert len(set(l.tolist())) == 10 and (d == 0).all()
    ix = oracle.OracleIndex(GOLD / "empty.idx")
    l, d = ix.search_batch(np.zeros((1, 8), dtype=np.float32), 3, 10)
    _same(l, d, arr["empty_labels"], arr["empty_dists"])
    small = np.load(GOLD / "small_data.npz")
    ix = oracle.OracleIndex(GOLD / "five.idx")
    l, d = ix.search(small["five"][0], 50, 1)
    _same(l, d, arr["five_labels"], arr["five_dists"])
    ix = oracle.OracleIndex(GOLD / "alldeleted.idx")
    l, d = ix.search(small["all20"][0], 5, 10)
    assert l.size == 0 and arr["alldeleted_labels"].size == 0
    ix = oracle.OracleIndex(GOLD / "collinear.idx")
    bcol = np.full(128, 0.5, dtype=np.float32)
    bcol[0] = 0.0
    l, d = ix.search(bcol, 100, 200)
    _same(l, d, arr["collinear_all_labels"], arr["collinear_all_dists"])
    allow = np.zeros(2, dtype=np.uint64)
    allow[0] = np.uint64(1 << 7)
    allow[1] = np.uint64(1 << (99 - 64))
    l, d = ix.search(bcol, 10, 64, filt=(allow, 100))
    _same(l, d, arr["collinear_f_labels"], arr["collinear_f_dists"])
    ix = oracle.OracleIndex(GOLD / "labels.idx")
    ql = np.load(GOLD / "labels_queries.npy")
    l, d = ix.search_batch(ql, 5, 0)
    _same(l, d, arr["labels_u_labels"], arr["labels_u_dists"])
    import workloads

    fw = workloads.mask_to_words(np.arange(2000) % 2 == 0)
    l, d = ix.search_batch(ql, 5, 20, filters=[(fw, 2000)])
    _same(l, d, arr["labels_f_labels"], arr["labels_f_dists"])


def test_config1_search_batch(oracle, golden, graphs):
    meta, arr = golden
    p = graphs.path("c1")
    assert sha256(p) == meta["cases"]["c1"]["index_sha"]
    _, q, *_ = graphs.data("c1")
    ix = oracle.OracleIndex(p)
    for ef in meta["cases"]["c1"]["efs"]:
        l, d = ix.search_batch(q, 10, ef)
        _same(l, d, arr[f"c1_ef{ef}_labels"], arr[f"c1_ef{ef}_dists"])


def test_cosine_filters_deletes(oracle, golden, graphs):
    meta, arr = golden
    import workloads

    case = meta["cases"]["c3s"]
    p = graphs.path("c3s", deleted=True)
    assert sha256(p) == case["deleted_index_sha"]
    _, q, *_ = graphs.data("c3s")
    ix = oracle.OracleIndex(p)
    fw = workloads.label_filter_bits(case["n"], lambda l: l % 10 == 0)
    for k, ef, filtered in case["groups"]:
        l, d = ix.search_batch(q, k, ef, filters=[(fw, case["n"])] if filtered else None)
        key = f"c3s_k{k}_ef{ef}_{'f' if filtered else 'u'}"
        _same(l, d, arr[key + "_labels"], arr[key + "_dists"])
    ix0 = oracle.OracleIndex(graphs.path("c3s"))
    l, d = ix0.search_batch(q, 10, 40)
    _same(l, d, arr["c3s_nodel_k10_ef40_labels"], arr["c3s_nodel_k10_ef40_dists"])


def test_highdim_and_inner_product(oracle, golden, graphs):
    meta, arr = golden
    _, q4, *_ = graphs.data("c4s")
    ix = oracle.OracleIndex(graphs.path("c4s"))
    for ef in meta["cases"]["c4s"]["efs"]:
        l, d = ix.search_batch(q4, 10, ef)
        _same(l, d, arr[f"c4s_ef{ef}_labels"], arr[f"c4s_ef{ef}_dists"])
    _, qip, *_ = graphs.data("ip")
    ix = oracle.OracleIndex(graphs.path("ip"))
    l, d = ix.search_batch(qip, 10, 100)
    _same(l, d, arr["ip_labels"], arr["ip_dists"])


def test_bruteforce(oracle, golden, graphs):
    _, arr = golden
    import workloads

    base, q, *_ = graphs.data("c1")
    l, d = oracle.bruteforce(base, q[:200], 10, "l2")
    _same(l, d, arr["c1_bf_labels"], arr["c1_bf_dists"])
    base3, q3, *_ = graphs.data("c3s")
    fw = workloads.label_filter_bits(4000, lambda x: x % 10 == 0)
    l, d = oracle.bruteforce(base3, q3[:100], 10, "cosine", filt=(fw, 4000))
    _same(l, d, arr["c3s_bf_f_labels"], arr["c3s_bf_f_dists"])
    base4, q4, *_ = graphs.data("c4s")
    l, d = oracle.bruteforce(base4, q4[:50], 10, "l2")
    _same(l, d, arr["c4s_bf_labels"], arr["c4s_bf_dists"])


def test_loader_rejects_what_the_reference_rejects(oracle, golden, tmp_path):
    meta, _ = golden
    fz = meta["fuzz"]
    src = (GOLD / fz["file"]).read_bytes()
    bad = tmp_path / "bad.idx"
    assert len(fz["flips"]) == fz["flips_tried"] and len(fz["cuts"]) == fz["cuts_tried"]
    for pos, bit in fz["flips"]:
        b = bytearray(src)
        b[pos] ^= 1 << bit
        bad.write_bytes(bytes(b))
        with pytest.raises(oracle.OracleError):
            oracle.OracleIndex(bad)
    for c in fz["cuts"]:
        bad.write_bytes(src[:c])
        with pytest.raises(oracle.OracleError):
            oracle.OracleIndex(bad)
    bad.write_bytes(src + b"\0")
    with pytest.raises(oracle.OracleError):
        oracle.OracleIndex(bad)
