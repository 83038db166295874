"""Compressed-precision batches route restrictive filters to an exact
tensor-core scan -- the rows the filter allows (mma.sync tiles of 8 queries)
or every row (the tcgen05 GEMM): those queries must return the exact k
nearest allowed, live rows (distances bit-identical to the graph's), and
every other query must be answered exactly as without routing."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _mask(n, fn):
    return np.asarray([bool(fn(i)) for i in range(n)])


MODES = ("auto", "allowed_rows", "every_row")


@pytest.mark.parametrize("mode", MODES)
def test_routed_queries_are_exact_knn_of_allowed_live_rows(hg, oracle, graphs, mode):
    import workloads

    base, q, *_ = graphs.data("c1")  # integer rows, d = 128 = padded width: every order is exact
    n = base.shape[0]
    ix = hg.Index.load(graphs.path("c1"))
    dead = [5, 77, 1234, 19999] + list(range(100, 20000, 997))
    for lab in dead:
        ix.mark_deleted(int(lab))
    rare = _mask(n, lambda i: i % 20 == 0)       # 5%: routed at filter_scan = 0.1
    common = _mask(n, lambda i: i % 2 == 0)      # 50%: walked
    fsel = np.where(np.arange(q.shape[0]) % 3 == 0, 0, np.where(np.arange(q.shape[0]) % 3 == 1, 1, -1))
    filters = [rare, common]
    walked = ix.search_batch_ex(q, 10, 80, filters=filters, filter_of_query=fsel, precision=2)
    routed = ix.search_batch_ex(q, 10, 80, filters=filters, filter_of_query=fsel, precision=2, filter_scan=0.1,
                                filter_scan_mode=mode)
    live_rare = rare.copy()
    live_rare[dead] = False
    sel = fsel == 0
    ol, od = oracle.bruteforce(base, q[sel], 10, "l2", filt=(workloads.mask_to_words(live_rare), n))
    np.testing.assert_array_equal(routed["label"][sel], ol)
    assert routed["distance"][sel].tobytes() == od.tobytes()
    np.testing.assert_array_equal(routed["label"][~sel], walked["label"][~sel])
    assert routed["distance"][~sel].tobytes() == walked["distance"][~sel].tobytes()
    # FP32 batches are never routed
    plain = ix.search_batch_ex(q, 10, 80, filters=filters, filter_of_query=fsel)
    np.testing.assert_array_equal(ix.search_batch_ex(q, 10, 80, filters=filters, filter_of_query=fsel,
                                                     filter_scan=0.1)["label"], plain["label"])


def test_server_routes_restrictive_filters(hg, graphs):
    base, q, *_ = graphs.data("c1")
    n = base.shape[0]
    ix = hg.Index.load(graphs.path("c1"))
    rare = _mask(n, lambda i: i % 25 == 3)
    reqs = [(q[i:i + 7], 10 if i % 2 else 3, 64, rare if i % 3 == 0 else None) for i in range(0, 700, 7)]
    srv = hg.Server(ix, precision=2, filter_scan=0.1, max_batch_queries=64)
    _, outs = srv.replay(reqs, np.zeros(len(reqs)))
    srv.close()
    for (qq, k, ef, f), got in zip(reqs, outs):
        want = ix.search_batch_ex(qq, k, ef, filters=[f] if f is not None else None, precision=2, filter_scan=0.1)
        np.testing.assert_array_equal(got["label"], want["label"])
        assert got["distance"].tobytes() == want["distance"].tobytes()


def _float_index(hg, n=6000, d=128, seed=7):
    r = np.random.default_rng(seed)
    centers = r.normal(0.0, 3.0, size=(40, d))
    base = (centers[r.integers(0, 40, n)] + r.normal(0.0, 1.0, size=(n, d))).astype(np.float32)
    q = (centers[r.integers(0, 40, 400)] + r.normal(0.0, 1.0, size=(400, d))).astype(np.float32)
    ix = hg.Index(d, "l2", 16, 100)
    ix.add(base)
    return ix, base, q


@pytest.mark.parametrize("mode", ("allowed_rows", "every_row"))
def test_routed_scan_exact_on_float_rows_with_mixed_k(hg, oracle, mode):
    """Float rows (the FP16 scores carry rounding error, so the answer rests on
    the margin), per-query k, deletes, a filter that allows nothing and one
    that allows fewer rows than k, runs of one filter that cross the 8-query
    tiles: every routed query gets the oracle's exact filtered k-NN."""
    import workloads

    ix, base, q = _float_index(hg)
    n = base.shape[0]
    dead = np.arange(3, n, 41)
    for lab in dead:
        ix.mark_deleted(int(lab))
    r = np.random.default_rng(3)
    masks = [r.random(n) < 0.06, r.random(n) < 0.03, np.zeros(n, bool), np.isin(np.arange(n), [5, 9, 300, 301, 4000])]
    fsel = np.full(q.shape[0], -1, np.int32)
    runs = [(0, 9), (1, 17), (2, 3), (3, 5), (0, 1), (1, 8), (0, 40)]
    at = 0
    for f, ln in runs:
        fsel[at:at + ln] = f
        at += 2 * ln  # unfiltered (walked) queries between the runs
    ks = r.choice(np.array([1, 10, 50]), q.shape[0]).astype(np.uint32)
    got = ix.search_batch_ex(q, 50, 96, k_per_query=ks, filters=masks, filter_of_query=fsel, precision=1,
                             filter_scan=0.1, filter_scan_mode=mode)
    for f, m in enumerate(masks):
        live = m.copy()
        live[dead] = False
        for kk in (1, 10, 50):
            sel = np.flatnonzero((fsel == f) & (ks == kk))
            if sel.size == 0:
                continue
            ol, od = oracle.bruteforce(base, q[sel], kk, "l2", filt=(workloads.mask_to_words(live), n))
            np.testing.assert_array_equal(got["label"][sel, :kk], ol, err_msg=f"filter {f} k {kk}")
            assert got["distance"][sel, :kk].tobytes() == od.tobytes(), f"filter {f} k {kk}"


def test_routed_scan_modes_agree_at_size(hg):
    """Both scans give the same rows on a batch where each routed query has
    its own k and many queries share a filter (several tiles per filter)."""
    ix, base, q = _float_index(hg, n=12000, seed=11)
    n = base.shape[0]
    r = np.random.default_rng(4)
    masks = [r.random(n) < 0.02 * (i + 1) for i in range(4)]
    fsel = r.integers(-1, 4, q.shape[0]).astype(np.int32)
    ks = r.choice(np.array([1, 10, 100]), q.shape[0]).astype(np.uint32)
    out = {}
    for mode in ("allowed_rows", "every_row"):
        out[mode] = ix.search_batch_ex(q, 100, 128, k_per_query=ks, filters=masks, filter_of_query=fsel,
                                       precision=2, filter_scan=0.1, filter_scan_mode=mode)
    routed = fsel >= 0
    for i in np.flatnonzero(routed):
        kk = ks[i]
        np.testing.assert_array_equal(out["allowed_rows"]["label"][i, :kk], out["every_row"]["label"][i, :kk])
        assert out["allowed_rows"]["distance"][i, :kk].tobytes() == out["every_row"]["distance"][i, :kk].tobytes()


def test_filter_scan_mode_is_validated(hg, graphs):
    ix = hg.Index.load(graphs.path("c1"))
    with pytest.raises(ValueError):
        ix.search_batch_ex(np.zeros((1, 128), np.float32), 1, 16, precision=2, filter_scan=0.1,
                           filter_scan_mode="rows")


def test_routed_every_row_seeded_large_k(hg, oracle, graphs):
    """2,100 routed queries at k = 100 over every row: the scan's thresholds
    are seeded by the bound pass; answers are the exact k nearest allowed,
    live rows."""
    import workloads

    base, q, *_ = graphs.data("c1")
    n = base.shape[0]
    ix = hg.Index.load(graphs.path("c1"))
    for lab in (3, 4000, 12345):
        ix.mark_deleted(lab)
    rare = _mask(n, lambda i: i % 16 == 5)
    qq = np.concatenate([q, q, q[:100]])
    out = ix.search_batch_ex(qq, 100, 128, filters=[rare], filter_of_query=np.zeros(qq.shape[0], np.int32),
                             precision=2, filter_scan=0.1, filter_scan_mode="every_row")
    live = rare.copy()
    live[[3, 4000, 12345]] = False
    ol, od = oracle.bruteforce(base, qq, 100, "l2", filt=(workloads.mask_to_words(live), n))
    np.testing.assert_array_equal(out["label"], ol)
    assert out["distance"].tobytes() == od.tobytes()
