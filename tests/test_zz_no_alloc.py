"""The allocation-free batch entry point (hg_index_search_batch_noalloc).

It exists for callers that cannot call cudaMalloc while they search; its
scratch is a static device array.  Its answers must equal those of the
allocating entry point, on two calls in a row (the array keeps the previous
call's contents), through the C ABI.  Collected last on purpose.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(hg, ix, q, k, ef, torch):
    d_q = torch.from_numpy(np.ascontiguousarray(q, dtype=np.float32)).cuda()
    d_out = torch.full((q.shape[0] * k * 4,), -1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    ix.search_noalloc(d_q.data_ptr(), q.shape[0], k, ef, d_out.data_ptr(), stream)
    torch.cuda.synchronize()
    return d_out.cpu().numpy().view(hg.NEIGHBOR).reshape(q.shape[0], k)


def test_no_alloc_batches_match_the_allocating_entry_point(hg, graphs):
    torch = pytest.importorskip("torch")
    _, q, *_ = graphs.data("c1")
    ix = hg.Index.load(graphs.path("c1"))
    want = ix.search_raw(q, 10, 40)  # allocating path; also mirrors the graph on the GPU
    for _ in range(2):  # second call reuses the static scratch left by the first
        got = _run(hg, ix, q, 10, 40, torch)
        np.testing.assert_array_equal(got["label"], want["label"])
        assert got["distance"].tobytes() == want["distance"].tobytes()


def test_no_alloc_cosine_with_deletes_and_limits(hg, graphs):
    torch = pytest.importorskip("torch")
    _, q, *_ = graphs.data("c3s")
    ix = hg.Index.load(graphs.path("c3s", deleted=True))
    want = ix.search_raw(q, 100, 400)
    for _ in range(2):
        got = _run(hg, ix, q, 100, 400, torch)
        np.testing.assert_array_equal(got["label"], want["label"])
        assert got["distance"].tobytes() == want["distance"].tobytes()
    with pytest.raises(ValueError, match="ef"):
        _run(hg, ix, q[:2], 10, 600, torch)


def test_no_alloc_overflow_reruns_match(hg, graphs):
    """Nine in ten nodes deleted and ef = 512: the filtered walk's candidate
    queue outgrows the 2,048-key spill pool, so queries go to the one-warp
    rerun pass; answers still equal the allocating path's bit for bit."""
    torch = pytest.importorskip("torch")
    _, q, *_ = graphs.data("c1")
    ix = hg.Index.load(graphs.path("c1"))
    for lab in range(20000):
        if lab % 10:
            ix.mark_deleted(lab)
    want = ix.search_raw(q[:64], 10, 512)
    for _ in range(2):
        got = _run(hg, ix, q[:64], 10, 512, torch)
        np.testing.assert_array_equal(got["label"], want["label"])
        assert got["distance"].tobytes() == want["distance"].tobytes()
    _, cnt = ix.search_batch_ex(q[:64], 10, 512, counters=True, pool_cap=2048)
    assert (cnt[:, 7] & 4).any(), "no query needed the rerun pass with a 2,048-key pool"


def test_no_alloc_needs_a_mirrored_graph(hg, graphs):
    torch = pytest.importorskip("torch")
    _, q, *_ = graphs.data("c1")
    fresh = hg.Index.load(graphs.path("c1"))
    with pytest.raises(RuntimeError, match="not mirrored"):
        _run(hg, fresh, q[:4], 10, 40, torch)
