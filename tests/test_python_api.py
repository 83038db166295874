"""The Python module against the reference's Python binding semantics
(python/bindings.cpp:114-233): argument conversion and errors, ids with -1
padding, the filter kinds, deletes, save / load, threads.  Searches run on
the GPU (marked); argument handling and empty indexes need none."""
from __future__ import annotations

import threading

import numpy as np
import pytest

gpu = pytest.mark.gpu


def _clustered(n, d, seed, clusters=16):
    # the reference's Python-test recipe: N(0, 4^2) centres, unit noise
    r = np.random.default_rng(seed)
    centers = r.normal(0, 4, size=(clusters, d))
    c = r.integers(0, clusters, size=n)
    return (centers[c] + r.normal(size=(n, d))).astype(np.float32)


def _exact(base, q, k, metric="l2"):
    if metric == "l2":
        d = ((q[:, None, :] - base[None, :, :]) ** 2).sum(-1)
    else:
        b = base / np.linalg.norm(base, axis=1, keepdims=True) if metric == "cosine" else base
        qq = q / np.linalg.norm(q, axis=1, keepdims=True) if metric == "cosine" else q
        d = -qq @ b.T
    return np.argsort(d, axis=1, kind="stable")[:, :k]


def _recall(got, truth):
    return np.mean([len(set(g[g >= 0]) & set(t)) / len(t) for g, t in zip(got, truth)])


@pytest.fixture(scope="module")
def small(hg):
    base = _clustered(3000, 32, 1)
    ix = hg.Index(dim=32)
    ix.add(base, num_threads=1)
    return ix, base, _clustered(100, 32, 2)


# ---- no GPU needed -----------------------------------------------------------

def test_properties_and_repr(hg):
    ix = hg.Index(dim=32)
    ix.add(_clustered(50, 32, 3))
    assert len(ix) == 50 and ix.dim == 32 and ix.metric == "l2" and ix.M == 16 and ix.ef_construction == 200
    assert not ix.read_only and 0 in ix and 49 in ix and 50 not in ix
    assert "Index dim=32" in repr(ix)
    assert hg.simd_isa() in {"scalar", "avx2", "avx512", "neon"}


def test_empty_index_search_pads(hg):
    ix = hg.Index(dim=3)
    ids, dists = ix.search(np.zeros(3, np.float32), k=2)
    assert ids.shape == (2,) and (ids == -1).all() and np.isinf(dists).all()


def test_argument_errors(hg):
    ix = hg.Index(dim=8)
    with pytest.raises(ValueError, match="shape"):
        ix.search(np.zeros((3, 7), np.float32))
    with pytest.raises(ValueError):
        ix.search(np.zeros((2, 2, 8), np.float32))
    with pytest.raises(ValueError, match="k must be"):
        ix.search(np.zeros(8, np.float32), k=0)
    with pytest.raises(TypeError):
        ix.search(np.array(["a", "b"]))
    with pytest.raises(ValueError):
        ix.add(np.zeros((4, 7), np.float32))
    with pytest.raises(ValueError, match="warps_per_query"):
        ix.search_batch_ex(np.zeros((1, 8), np.float32), 1, precision=2, warps_per_query=2)
    with pytest.raises(ValueError, match="rerank_factor"):
        ix.search_batch_ex(np.zeros((1, 8), np.float32), 1, precision=2, rerank_factor=-1)
    with pytest.raises(ValueError, match="warps_per_query"):
        hg.Server(ix, precision=2, warps_per_query=8)
    for bad in (dict(dim=0), dict(dim=8, metric="hamming"), dict(dim=8, M=1)):
        with pytest.raises(ValueError):
            hg.Index(**bad)


def test_id_errors(hg):
    ix = hg.Index(dim=4)
    v = np.random.default_rng(0).random((3, 4), dtype=np.float32)
    with pytest.raises(ValueError, match="non-negative"):
        ix.add(v, ids=[1, -2, 3])
    with pytest.raises(ValueError, match="shape"):
        ix.add(v, ids=[1, 2])
    with pytest.raises(TypeError):
        ix.add(v, ids=[1.5, 2.5, 3.5])
    with pytest.raises(ValueError, match="duplicate"):
        ix.add(v, ids=[1, 1, 2])
    ix.add(v, ids=[1, 2, 3])
    with pytest.raises(ValueError, match="already exists"):
        ix.add(v[:1], ids=[2])
    assert len(ix) == 3


def test_get_vector_normalises_cosine_and_keeps_caller_buffer(hg):
    v = np.array([[3.0, 4.0]], np.float32)
    ix = hg.Index(dim=2, metric="cosine")
    ix.add(v)
    np.testing.assert_allclose(ix.get_vector(0), [0.6, 0.8], rtol=1e-6)
    np.testing.assert_array_equal(v, [[3.0, 4.0]])


def test_filter_type_errors(hg):
    ix = hg.Index(dim=4)
    ix.add(np.eye(4, dtype=np.float32))
    with pytest.raises(TypeError):
        ix.search(np.ones((1, 4), np.float32), k=2, filter=np.array([0.5, 1.5]))
    with pytest.raises(TypeError):
        ix.search(np.ones((1, 4), np.float32), k=2, filter="nope")


# ---- on the GPU ----------------------------------------------------------------

@gpu
@pytest.mark.parametrize("metric", ["l2", "ip", "cosine"])
def test_recall_and_result_types(hg, metric):
    base, q = _clustered(2000, 24, 3), _clustered(50, 24, 4)
    ix = hg.Index(dim=24, metric=metric)
    ix.add(base)
    ids, dists = ix.search(q, k=10, ef=400 if metric == "ip" else 100)
    assert ids.shape == (50, 10) and ids.dtype == np.int64 and dists.dtype == np.float32
    assert np.all(np.diff(dists, axis=1) >= 0)
    assert _recall(ids, _exact(base, q, 10, metric)) >= (0.9 if metric == "ip" else 0.95)


@gpu
def test_single_query_and_padding(hg, small):
    ix, base, q = small
    ids, dists = ix.search(q[0], k=5)
    assert ids.shape == (5,) and dists.shape == (5,)
    np.testing.assert_array_equal(ids, ix.search(q[:1], k=5)[0][0])
    tiny = hg.Index(dim=4)
    tiny.add(np.eye(4, dtype=np.float32))
    ids, dists = tiny.search(np.ones((2, 4), np.float32), k=6)
    assert (ids[:, :4] >= 0).all() and (ids[:, 4:] == -1).all() and np.isinf(dists[:, 4:]).all()


@gpu
def test_dtype_and_layout_conversion(hg, small):
    ix, base, q = small
    want = ix.search(q[:10], k=5, ef=50)[0]
    np.testing.assert_array_equal(ix.search(np.asfortranarray(q[:10]), k=5, ef=50)[0], want)
    np.testing.assert_array_equal(ix.search(np.repeat(q[:10], 2, axis=0)[::2], k=5, ef=50)[0], want)
    np.testing.assert_array_equal(ix.search(q[:10].tolist(), k=5, ef=50)[0], want)
    np.testing.assert_array_equal(ix.search(q[:10].astype(np.float64), k=5, ef=50)[0], want)


@gpu
def test_custom_ids(hg):
    base = _clustered(300, 8, 5)
    ix = hg.Index(dim=8)
    ix.add(base[:100], ids=np.arange(1000, 1100))
    ix.add(base[100:200])  # arange(len, len + n) = 100..199
    assert 1000 in ix and 150 in ix and 99 not in ix
    ids, dists = ix.search(base[[5, 150]], k=1)
    assert ids[0, 0] == 1005 and ids[1, 0] == 150 and abs(float(dists[0, 0])) < 1e-5


@gpu
@pytest.mark.parametrize("kind", ["callable", "mask", "ids", "list"])
def test_filter_kinds(hg, small, kind):
    ix, base, q = small
    allowed = np.zeros(len(base), dtype=bool)
    allowed[::7] = True
    flt = {"callable": lambda label: bool(allowed[label]), "mask": allowed, "ids": np.flatnonzero(allowed),
           "list": np.flatnonzero(allowed).tolist()}[kind]
    ids, _ = ix.search(q[:30], k=10, ef=100, filter=flt)
    assert allowed[ids[ids >= 0]].all()
    truth = np.flatnonzero(allowed)[_exact(base[allowed], q[:30], 10)]
    assert _recall(ids, truth) >= 0.9


@gpu
def test_filter_callback_exception_propagates(hg, small):
    ix, _, q = small

    def bad(label):
        raise KeyError("boom")

    with pytest.raises(KeyError, match="boom"):
        ix.search(q[:4], k=3, filter=bad)


@gpu
def test_mark_deleted_and_save_load(hg, tmp_path):
    base = _clustered(1000, 16, 6)
    ix = hg.Index(dim=16)
    ix.add(base)
    for label in range(0, 1000, 2):
        ix.mark_deleted(label)
    ids, _ = ix.search(base[:20], k=10, ef=100)
    assert (ids[ids >= 0] % 2 == 1).all()
    p = tmp_path / "i.idx"
    ix.save(p)
    for mmap in (False, True):
        back = hg.Index.load(p, mmap=mmap)
        np.testing.assert_array_equal(back.search(base[:20], k=10, ef=100)[0], ids)
        assert back.is_deleted(0) and not back.is_deleted(1)


@gpu
def test_concurrent_searches_from_threads(hg, small):
    ix, _, q = small
    want = ix.search(q, k=10, ef=64)[0]
    errors, out = [], [None] * 6

    def run(i):
        try:
            out[i] = ix.search(q, k=10, ef=64)[0]
        except Exception as e:  # noqa: BLE001 - collected for the assertion below
            errors.append(e)

    ts = [threading.Thread(target=run, args=(i,)) for i in range(6)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert not errors
    for o in out:
        np.testing.assert_array_equal(o, want)
