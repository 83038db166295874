"""Compressed-precision batches route restrictive filters to the exact
tensor-core scan: those queries must return the exact k nearest allowed,
live rows (distances bit-identical to the graph's), and every other query
must be answered exactly as without routing."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _mask(n, fn):
    return np.asarray([bool(fn(i)) for i in range(n)])


def test_routed_queries_are_exact_knn_of_allowed_live_rows(hg, oracle, graphs):
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
    routed = ix.search_batch_ex(q, 10, 80, filters=filters, filter_of_query=fsel, precision=2, filter_scan=0.1)
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
