"""GPU parity: the CUDA query path against the reference's own results and
against the oracle, through the C ABI.

Bar: ids and distances bit-identical to the reference's search_batch on the
same graph (the kernels reproduce its AVX-512 summation order, so this holds
for float data as well as integer data), and per-query traversal counts
(lists read, distances computed, nodes visited) equal to the oracle's.
"""
from __future__ import annotations

import threading

import numpy as np
import pytest

from conftest import GOLD

pytestmark = pytest.mark.gpu


def _eq(rec, want_l, want_d, what=""):
    got_l = rec["label"].astype(np.int64)
    np.testing.assert_array_equal(got_l, want_l, err_msg=f"labels {what}")
    assert rec["distance"].astype(np.float32).tobytes() == want_d.astype(np.float32).tobytes(), f"distances {what}"


def _eq_oracle(rec, ol, od, what=""):
    np.testing.assert_array_equal(rec["label"], ol, err_msg=f"labels {what}")
    assert rec["distance"].tobytes() == od.tobytes(), f"distances {what}"


def test_config1_bitwise_vs_reference(hg, golden, graphs):
    meta, arr = golden
    _, q, *_ = graphs.data("c1")
    ix = hg.Index.load(graphs.path("c1"))
    for ef in meta["cases"]["c1"]["efs"]:
        rec = ix.search_raw(q, 10, ef)
        _eq(rec, arr[f"c1_ef{ef}_labels"], arr[f"c1_ef{ef}_dists"], f"ef={ef}")


def test_traversal_counts_equal_oracle(hg, oracle, graphs):
    _, q, *_ = graphs.data("c1")
    p = graphs.path("c1")
    ix = hg.Index.load(p)
    ox = oracle.OracleIndex(p)
    for ef in (10, 40, 160):
        rec, cnt = ix.search_batch_ex(q, 10, ef, counters=True)
        ol, od, oc = ox.search_batch(q, 10, ef, counters=True)
        _eq_oracle(rec, ol, od, f"ef={ef}")
        # upper lists, upper distances, layer-0 lists, layer-0 distances, visited, results
        for col in (0, 1, 2, 3, 4, 6):
            np.testing.assert_array_equal(cnt[:, col], oc[:, col], err_msg=f"counter {col} ef={ef}")


def test_cosine_filters_and_deletes_vs_reference(hg, golden, graphs):
    meta, arr = golden
    import workloads

    case = meta["cases"]["c3s"]
    _, q, *_ = graphs.data("c3s")
    ix = hg.Index.load(graphs.path("c3s", deleted=True))
    fw = workloads.label_filter_bits(case["n"], lambda l: l % 10 == 0)
    for k, ef, filtered in case["groups"]:
        rec = ix.search_raw(q, k, ef, filter=hg.Bitset(fw, case["n"]) if filtered else None)
        key = f"c3s_k{k}_ef{ef}_{'f' if filtered else 'u'}"
        _eq(rec, arr[key + "_labels"], arr[key + "_dists"], key)
    ix0 = hg.Index.load(graphs.path("c3s"))
    _eq(ix0.search_raw(q, 10, 40), arr["c3s_nodel_k10_ef40_labels"], arr["c3s_nodel_k10_ef40_dists"], "nodel")


def test_one_mixed_batch_equals_the_reference_groups(hg, golden, graphs):
    """Per-query k / ef / filter in one launch == one reference call per group."""
    meta, arr = golden
    import workloads

    case = meta["cases"]["c3s"]
    _, q, *_ = graphs.data("c3s")
    ix = hg.Index.load(graphs.path("c3s", deleted=True))
    fw = workloads.label_filter_bits(case["n"], lambda l: l % 10 == 0)
    groups = case["groups"]
    rows, efs, ks, fsel, keys = [], [], [], [], []
    for gi, (k, ef, filtered) in enumerate(groups):
        rows.append(q)
        efs += [ef] * q.shape[0]
        ks += [k] * q.shape[0]
        fsel += [0 if filtered else -1] * q.shape[0]
        keys.append(f"c3s_k{k}_ef{ef}_{'f' if filtered else 'u'}")
    allq = np.concatenate(rows)
    perm = np.random.default_rng(3).permutation(allq.shape[0])  # interleave the groups
    kmax = max(ks)
    rec = ix.search_batch_ex(allq[perm], kmax, ef_per_query=np.array(efs)[perm], k_per_query=np.array(ks)[perm],
                             filters=[hg.Bitset(fw, case["n"])], filter_of_query=np.array(fsel)[perm])
    back = np.empty_like(rec)
    back[perm] = rec
    nq = q.shape[0]
    for gi, key in enumerate(keys):
        k = ks[gi * nq]
        part = back[gi * nq:(gi + 1) * nq, :k]
        _eq(part, arr[key + "_labels"], arr[key + "_dists"], key + " (mixed)")
        assert (back[gi * nq:(gi + 1) * nq, k:]["label"] == hg.INVALID_LABEL).all()


def test_deletes_after_upload(hg, golden, graphs):
    meta, arr = golden
    import workloads

    case = meta["cases"]["c3s"]
    _, q, *_ = graphs.data("c3s")
    ix = hg.Index.load(graphs.path("c3s"))
    ix.search_raw(q[:4], 10, 40)  # graph now mirrored on the device
    for lab in workloads.random_deletes(case["n"], 0.01, seed=2):
        ix.mark_deleted(int(lab))
    rec = ix.search_raw(q, 10, 40)
    _eq(rec, arr["c3s_k10_ef40_u_labels"], arr["c3s_k10_ef40_u_dists"], "deleted after upload")


def test_highdim_and_inner_product_vs_reference(hg, golden, graphs):
    meta, arr = golden
    _, q4, *_ = graphs.data("c4s")
    ix = hg.Index.load(graphs.path("c4s"))
    for ef in meta["cases"]["c4s"]["efs"]:
        _eq(ix.search_raw(q4, 10, ef), arr[f"c4s_ef{ef}_labels"], arr[f"c4s_ef{ef}_dists"], f"c4s ef={ef}")
    _, qip, *_ = graphs.data("ip")
    ix = hg.Index.load(graphs.path("ip"))
    _eq(ix.search_raw(qip, 10, 100), arr["ip_labels"], arr["ip_dists"], "ip")


def test_edge_cases_vs_reference(hg, golden):
    _, arr = golden
    small = np.load(GOLD / "small_data.npz")
    r = hg.Index.load(GOLD / "dim1.idx").search_one(np.array([42.2], dtype=np.float32), 3, 50)
    _eq(r, arr["dim1_labels"], arr["dim1_dists"], "dim1")
    assert list(r["label"]) == [42, 43, 41]
    r = hg.Index.load(GOLD / "identical.idx").search_one(np.full(12, 0.5, dtype=np.float32), 10, 64)
    _eq(r, arr["identical_labels"], arr["identical_dists"], "identical")
    rec = hg.Index.load(GOLD / "empty.idx").search_raw(np.zeros((1, 8), dtype=np.float32), 3, 10)
    _eq(rec, arr["empty_labels"], arr["empty_dists"], "empty")
    r = hg.Index.load(GOLD / "five.idx").search_one(small["five"][0], 50, 1)  # k > size, ef < k
    _eq(r, arr["five_labels"], arr["five_dists"], "five")
    r = hg.Index.load(GOLD / "alldeleted.idx").search_one(small["all20"][0], 5, 10)
    assert r.size == 0
    col = hg.Index.load(GOLD / "collinear.idx")
    bcol = np.full(128, 0.5, dtype=np.float32)
    bcol[0] = 0.0
    r = col.search_one(bcol, 100, 200)
    _eq(r, arr["collinear_all_labels"], arr["collinear_all_dists"], "collinear all")
    r = col.search_one(bcol, 10, 64, filter=np.array([7, 99]))
    _eq(r, arr["collinear_f_labels"], arr["collinear_f_dists"], "collinear filter")
    lab = hg.Index.load(GOLD / "labels.idx")
    ql = np.load(GOLD / "labels_queries.npy")
    _eq(lab.search_raw(ql, 5, 0), arr["labels_u_labels"], arr["labels_u_dists"], "labels default ef")
    mask = np.arange(2000) % 2 == 0
    _eq(lab.search_raw(ql, 5, 20, filter=mask), arr["labels_f_labels"], arr["labels_f_dists"], "labels filtered")
    # a callable filter (FunctionFilter) gives the same answer as the bitset
    rec = lab.search_raw(ql, 5, 20, filter=lambda l: l % 2 == 0)
    _eq(rec, arr["labels_f_labels"], arr["labels_f_dists"], "labels predicate")


def test_tiers_keep_results_exact(hg, oracle, graphs):
    """Tiny hash / candidate head / spill pool force the global bitmap, the
    pool and the rerun pass; the answers must not change."""
    import workloads

    _, q, *_ = graphs.data("c3s")
    p = graphs.path("c3s", deleted=True)
    ix = hg.Index.load(p)
    ox = oracle.OracleIndex(p)
    fw = workloads.label_filter_bits(4000, lambda l: l % 10 == 0)
    fsel = np.where(np.arange(q.shape[0]) % 2 == 0, 0, -1)
    ol, od = ox.search_batch(q, 100, 400, filters=[(fw, 4000)], fsel=fsel)
    for shape in (dict(hash_slots=256), dict(cand_cap=128), dict(cand_cap=128, pool_cap=32),
                  dict(hash_slots=256, cand_cap=128, pool_cap=32, warps_per_block=1)):
        rec, cnt = ix.search_batch_ex(q, 100, 400, filters=[hg.Bitset(fw, 4000)], filter_of_query=fsel,
                                      counters=True, **shape)
        _eq_oracle(rec, ol, od, str(shape))
        tiers = np.bitwise_or.reduce(cnt[:, 7])
        if "hash_slots" in shape:
            assert tiers & 1, "bitmap tier not reached"
        if "pool_cap" in shape:
            assert tiers & 4, "rerun tier not reached"
        elif "cand_cap" in shape:
            assert tiers & 2, "spill pool not reached"


def test_second_pool_tier_keeps_results_exact(hg, oracle, tmp_path):
    """A 0.5%-density filter at ef=300 on 100,000 nodes: until 300 eligible
    results are found every visited node joins the candidate queue, which
    outgrows the 8K-key first pool tier; the queries must move to the second
    tier (not the rerun pass) and answer exactly as the oracle."""
    import workloads

    base, q = workloads.int_mixture(100_000, 16, 32, 48)
    ix = hg.Index(16, "l2", 8, 64)
    ix.add(base, num_threads=0)
    p = tmp_path / "tier2.idx"
    ix.save(p)
    ix = hg.Index.load(p)
    ox = oracle.OracleIndex(p)
    fw = workloads.label_filter_bits(100_000, lambda l: l % 200 == 0)
    fsel = np.zeros(q.shape[0], dtype=np.int32)
    ol, od, ocnt = ox.search_batch(q, 10, 300, filters=[(fw, 100_000)], fsel=fsel, counters=True)
    rec, cnt = ix.search_batch_ex(q, 10, 300, filters=[hg.Bitset(fw, 100_000)], filter_of_query=fsel, counters=True)
    _eq_oracle(rec, ol, od, "second pool tier")
    assert int(ocnt[:, 5].max()) > 8192, "workload too small to leave the first tier"
    assert (cnt[:, 7] & 8).any(), "second pool tier not reached"
    assert not (cnt[:, 7] & 4).any(), "rerun pass used"
    for col in (2, 3, 4, 6):  # layer-0 lists, distances, visited, results
        np.testing.assert_array_equal(cnt[:, col], ocnt[:, col], err_msg=f"counter {col}")


def test_batch_equals_sequential(hg, graphs):
    _, q, *_ = graphs.data("c1")
    ix = hg.Index.load(graphs.path("c1"))
    rec = ix.search_raw(q[:100], 5, 50)
    for i in range(100):
        r = ix.search_one(q[i], 5, 50)
        np.testing.assert_array_equal(r["label"], rec[i]["label"])


def test_concurrent_callers(hg, graphs):
    _, q, *_ = graphs.data("c1")
    ix = hg.Index.load(graphs.path("c1"))
    want = ix.search_raw(q, 10, 40)
    errs = []

    def run():
        try:
            for _ in range(3):
                got = ix.search_raw(q, 10, 40)
                if not np.array_equal(got["label"], want["label"]):
                    errs.append("mismatch")
        except Exception as e:  # noqa: BLE001
            errs.append(repr(e))

    ts = [threading.Thread(target=run) for _ in range(4)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert not errs, errs


def test_errors(hg, graphs):
    _, q, *_ = graphs.data("c1")
    ix = hg.Index.load(graphs.path("c1"))
    with pytest.raises(ValueError, match="k must be > 0"):
        ix.search_raw(q[:1], 0)
    with pytest.raises(ValueError):
        ix.search_batch_ex(q[:2], 5, k_per_query=[3, 9])  # per-query k above the row stride
    with pytest.raises(ValueError):
        ix.search_batch_ex(q[:2], 5, filters=[np.array([1, 2])], filter_of_query=[0, 3])


@pytest.mark.parametrize("dim", [37, 200, 256, 500, 700])
@pytest.mark.parametrize("metric", ["l2", "ip"])
def test_every_distance_layout_vs_oracle(hg, oracle, tmp_path, dim, metric):
    """Float Gaussian rows (summation order matters) at widths that use the
    runtime layouts (37, 200, 700) and the two-rows-per-pass layouts (256,
    500): ids and distances bit-identical to the oracle; the FP16 / FP8 paths'
    fused rerank returns the exact kernel's distances for the ids it keeps."""
    rng = np.random.default_rng(dim)
    base = rng.normal(size=(1500, dim)).astype(np.float32)
    q = rng.normal(size=(40, dim)).astype(np.float32)
    ix = hg.Index(dim, metric, 8, 64)
    ix.add(base, num_threads=0)
    p = tmp_path / "g.idx"
    ix.save(p)
    ix = hg.Index.load(p)
    ol, od = oracle.OracleIndex(p).search_batch(q, 10, 64)
    _eq_oracle(ix.search_batch_ex(q, 10, 64), ol, od, f"dim={dim} {metric}")
    pd = -(-dim // 16) * 16  # graph rows are zero-padded to a multiple of 16 and summed over pd
    qp = np.zeros((q.shape[0], pd), np.float32)
    qp[:, :dim] = q
    bp = np.zeros((base.shape[0], pd), np.float32)
    bp[:, :dim] = base
    for prec in (1, 2):
        rec = ix.search_batch_ex(q, 10, 64, precision=prec)
        for qi in range(q.shape[0]):
            for lab, dist in zip(rec["label"][qi], rec["distance"][qi]):
                # each returned distance is the exact FP32 distance of that id
                want = oracle.kernel("avx512", metric == "l2", qp[qi], bp[int(lab)])
                if metric != "l2":
                    want = np.float32(np.float32(1.0) - want)
                assert np.float32(dist).tobytes() == np.float32(want).tobytes(), f"dim={dim} prec={prec}"

