"""The continuous-batching server: requests of mixed k, ef and filters, many
batches in flight at once, each result identical to the same request run
alone through search_batch."""
from __future__ import annotations

import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _requests(q, n, seed, n_labels):
    r = np.random.default_rng(seed)
    reqs = []
    for _ in range(n):
        nq = int(r.integers(1, 40))
        rows = r.integers(0, q.shape[0], nq)
        k = int(r.choice([1, 10, 50]))
        ef = int(r.choice([0, 16, 48, 96, 128]))
        f = None
        if r.random() < 0.3:
            f = r.random(n_labels) < 0.1
        reqs.append((q[rows], k, ef, f))
    return reqs


@pytest.mark.parametrize("precision", [0, 2])
def test_same_result_alone_and_in_the_mix(hg, graphs, precision):
    base, q, *_ = graphs.data("c1")
    ix = hg.Index.load(graphs.path("c1"))
    reqs = _requests(q, 90, 5, base.shape[0])
    alone = [ix.search_batch_ex(qq, k, ef, filters=[f] if f is not None else None, precision=precision)
             for (qq, k, ef, f) in reqs]
    srv = hg.Server(ix, max_inflight=4, max_batch_queries=96, precision=precision)
    results = [None] * len(reqs)

    def worker(part):
        tickets = [(i, srv.submit(*reqs[i])) for i in part]
        for i, t in tickets:
            results[i] = srv.wait(t)

    threads = [threading.Thread(target=worker, args=(list(range(j, len(reqs), 3)),)) for j in range(3)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    for i, (got, lat) in enumerate(results):
        assert lat >= 0
        np.testing.assert_array_equal(got["label"], alone[i]["label"], err_msg=f"request {i}")
        assert got["distance"].tobytes() == alone[i]["distance"].tobytes()
    srv.close()


def test_replay_open_loop_statistics(hg, graphs):
    base, q, *_ = graphs.data("c1")
    ix = hg.Index.load(graphs.path("c1"))
    reqs = _requests(q, 200, 6, base.shape[0])
    arrivals = np.cumsum(np.random.default_rng(7).exponential(1e-4, len(reqs)))
    srv = hg.Server(ix, max_inflight=4, max_batch_queries=128)
    stats, outs = srv.replay(reqs, arrivals)
    assert stats["requests"] == len(reqs)
    assert stats["queries"] == sum(r[0].shape[0] for r in reqs)
    assert 0 < stats["p50_ms"] <= stats["p99_ms"] <= stats["p999_ms"] <= stats["max_ms"]
    assert stats["batches"] >= 2
    for (qq, k, ef, f), got in zip(reqs[:20], outs[:20]):
        want = ix.search_batch_ex(qq, k, ef, filters=[f] if f is not None else None)
        np.testing.assert_array_equal(got["label"], want["label"])
    srv.close()


def test_bad_requests_fail_cleanly(hg, graphs):
    base, q, *_ = graphs.data("c1")
    ix = hg.Index.load(graphs.path("c1"))
    srv = hg.Server(ix)
    with pytest.raises(ValueError):
        srv.submit(q[:2], 0)
    t = srv.submit(q[:2], 5, 20)
    got, _ = srv.wait(t)
    assert got.shape == (2, 5)
    with pytest.raises(ValueError):
        srv.wait(t)  # already collected
    srv.close()
