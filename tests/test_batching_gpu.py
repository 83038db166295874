"""Batching addition: CUDA-graph replay of device-resident batches and the
launch-shape autotuner.  Neither may change an answer: every result is
compared bit for bit with the plain host-path search."""
from __future__ import annotations

import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev_batch(torch, ix, hg, q, k, efs, graph, reps):
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(device=dev)
    q_d = torch.from_numpy(q).to(dev)
    ef_d = torch.from_numpy(efs.astype(np.int32)).to(dev)
    out_d = torch.empty((q.shape[0], k, 4), dtype=torch.int32, device=dev)
    outs = []
    for _ in range(reps):
        out_d.zero_()
        torch.cuda.synchronize()
        ix.search_device(q_d.data_ptr(), q.shape[0], k, int(efs.max()), out_d.data_ptr(), stream.cuda_stream,
                         ef_ptr=ef_d.data_ptr(), graph=graph)
        torch.cuda.synchronize()
        outs.append(out_d.cpu().numpy().view(hg.NEIGHBOR).reshape(q.shape[0], k).copy())
    return outs, (q_d, ef_d, out_d, stream)


def test_graph_replay_equals_host_path(hg, graphs):
    torch = pytest.importorskip("torch")
    base, q, *_ = graphs.data("c1")
    ix = hg.Index.load(graphs.path("c1"))
    efs = np.random.default_rng(3).choice(np.array([10, 20, 40, 80, 160], dtype=np.uint32), q.shape[0])
    want = ix.search_batch_ex(q, 10, ef_per_query=efs)
    outs, (q_d, ef_d, out_d, stream) = _dev_batch(torch, ix, hg, q, 10, efs, graph=True, reps=4)
    for i, got in enumerate(outs):  # plain run, capture + launch, two replays
        np.testing.assert_array_equal(got["label"], want["label"], err_msg=f"call {i}")
        assert got["distance"].tobytes() == want["distance"].tobytes()
    # the graph reads its inputs at replay time: new query values, same buffer
    q2 = np.ascontiguousarray(q[::-1])
    q_d.copy_(torch.from_numpy(q2).to(q_d.device))
    out_d.zero_()
    torch.cuda.synchronize()
    ix.search_device(q_d.data_ptr(), q.shape[0], 10, int(efs.max()), out_d.data_ptr(), stream.cuda_stream,
                     ef_ptr=ef_d.data_ptr(), graph=True)
    torch.cuda.synchronize()
    got = out_d.cpu().numpy().view(hg.NEIGHBOR).reshape(q.shape[0], 10)
    np.testing.assert_array_equal(got["label"], ix.search_batch_ex(q2, 10, ef_per_query=efs)["label"])


def test_graph_follows_tombstones(hg, graphs):
    torch = pytest.importorskip("torch")
    base, q, *_ = graphs.data("c1")
    ix = hg.Index.load(graphs.path("c1"))
    efs = np.full(q.shape[0], 40, dtype=np.uint32)
    _dev_batch(torch, ix, hg, q, 10, efs, graph=True, reps=3)  # graph captured
    first = ix.search_batch_ex(q[:1], 1, 40)["label"][0, 0]
    ix.mark_deleted(int(first))
    outs, _ = _dev_batch(torch, ix, hg, q, 10, efs, graph=True, reps=3)
    want = ix.search_batch_ex(q, 10, ef_per_query=efs)
    for got in outs:
        np.testing.assert_array_equal(got["label"], want["label"])
    assert int(first) not in set(outs[-1]["label"].ravel().tolist())


def test_autotune_keeps_answers(hg, graphs, tmp_path):
    base, q, *_ = graphs.data("c1")
    ix = hg.Index.load(graphs.path("c1"))
    efs = np.random.default_rng(5).choice(np.array([10, 40, 100, 160], dtype=np.uint32), q.shape[0])
    before = ix.search_batch_ex(q, 10, ef_per_query=efs)
    sample = np.random.default_rng(9).permutation(q)[:256]
    path = tmp_path / "tune.json"
    table = ix.autotune(sample, k=10, ef_max=160, precision=0, path=path)
    his = [e["ef_hi"] for e in table["entries"]]
    assert his == [16, 32, 64, 96, 128, 192]
    for e in table["entries"]:
        assert e["us_per_query"] <= e["default_us_per_query"] + 1e-9
    after = ix.search_batch_ex(q, 10, ef_per_query=efs)
    np.testing.assert_array_equal(after["label"], before["label"])
    assert after["distance"].tobytes() == before["distance"].tobytes()
    # a fresh index takes the saved table
    ix2 = hg.Index.load(graphs.path("c1"))
    ix2.set_tuning(path)
    np.testing.assert_array_equal(ix2.search_batch_ex(q, 10, ef_per_query=efs)["label"], before["label"])
    with pytest.raises(ValueError):
        ix2.set_tuning(json.dumps({"entries": [{"precision": 0, "ef_hi": 16, "hash_slots": 300, "cand_cap": 128,
                                               "warps_per_block": 1}]}))


def test_single_launch_and_mixed_tuning_keep_answers(hg, graphs):
    """One largest-ef-first launch over all buckets, and the mixed-batch
    tuner (which may choose it), answer exactly like the per-bucket launches."""
    base, q, *_ = graphs.data("c1")
    ix = hg.Index.load(graphs.path("c1"))
    efs = np.random.default_rng(6).choice(np.array([10, 20, 40, 80, 160], dtype=np.uint32), q.shape[0])
    ks = np.random.default_rng(7).choice(np.array([1, 5, 10], dtype=np.uint32), q.shape[0])
    before = ix.search_batch_ex(q, 10, ef_per_query=efs, k_per_query=ks)
    single = {"launch_mode": 1, "entries": [{"precision": 0, "ef_hi": 192, "hash_slots": 512, "cand_cap": 224,
                                             "warps_per_block": 2}]}
    ix.set_tuning(json.dumps(single))
    got = ix.search_batch_ex(q, 10, ef_per_query=efs, k_per_query=ks)
    np.testing.assert_array_equal(got["label"], before["label"])
    assert got["distance"].tobytes() == before["distance"].tobytes()
    sample = np.random.default_rng(9).permutation(q)[:512]
    table = ix.autotune(sample, k=10, ef_max=160, ef_per_query=efs[:512])
    assert table["launch_mode"] in (0, 1)
    got = ix.search_batch_ex(q, 10, ef_per_query=efs, k_per_query=ks)
    np.testing.assert_array_equal(got["label"], before["label"])
    assert got["distance"].tobytes() == before["distance"].tobytes()
