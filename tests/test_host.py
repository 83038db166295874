"""Host-side behaviour of libhnswgpu that needs no GPU: the C ABI exports,
the CPU graph builder (byte-identical to the reference's), FORMAT v1 loading
and its rejections, accessors and argument errors."""
from __future__ import annotations

import ctypes
import re

import numpy as np
import pytest

from conftest import GOLD, REPO, sha256


def _declared(header):
    text = (REPO / "include" / header).read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(hgd?_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_entry_point(hg):
    lib = ctypes.CDLL(str(hg.LIB_PATH))
    names = _declared("hnswgpu.h") + _declared("hnswgpu_device.h")
    assert len(names) > 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_builder_bytes_match_reference(golden, graphs):
    meta, _ = golden
    for name in ("c1", "c3s", "c4s", "ip"):
        assert sha256(graphs.path(name)) == meta["cases"][name]["index_sha"], name
    assert sha256(graphs.path("c3s", deleted=True)) == meta["cases"]["c3s"]["deleted_index_sha"]


def test_load_save_round_trip_is_byte_identical(hg, golden, tmp_path):
    meta, _ = golden
    for name, h in meta["small"].items():
        for mmap in (False, True):
            ix = hg.Index.load(GOLD / f"{name}.idx", mmap)
            assert ix.read_only == mmap
            out = tmp_path / f"{name}_{int(mmap)}.idx"
            ix.save(out)
            assert sha256(out) == h, (name, mmap)


def test_loader_rejects_what_the_reference_rejects(hg, golden, tmp_path):
    meta, _ = golden
    fz = meta["fuzz"]
    src = (GOLD / fz["file"]).read_bytes()
    bad = tmp_path / "bad.idx"
    for pos, bit in fz["flips"]:
        b = bytearray(src)
        b[pos] ^= 1 << bit
        bad.write_bytes(bytes(b))
        for mmap in (False, True):
            with pytest.raises(RuntimeError, match="corrupt or incompatible|empty file|cannot"):
                hg.Index.load(bad, mmap)
    for c in fz["cuts"]:
        bad.write_bytes(src[:c])
        for mmap in (False, True):
            with pytest.raises(RuntimeError):
                hg.Index.load(bad, mmap)
    bad.write_bytes(src + b"\0")
    with pytest.raises(RuntimeError):
        hg.Index.load(bad, False)
    with pytest.raises(RuntimeError):
        hg.Index.load(tmp_path / "missing.idx", False)
    with pytest.raises(RuntimeError):
        hg.Index.load(tmp_path / "missing.idx", True)


def test_accessors_follow_the_reference(hg):
    ix = hg.Index.load(GOLD / "labels.idx")
    assert len(ix) == 300 and ix.dim == 6 and ix.metric == "cosine" and ix.M == 6
    assert ix.ef == 33 and ix.ef_construction == 40 and not ix.read_only
    assert 1000 in ix and 1003 in ix and 1001 not in ix
    assert ix.is_deleted(1003) and not ix.is_deleted(1000) and not ix.is_deleted(-1)
    v = ix.get_vector(1000)
    assert v.shape == (6,) and abs(float(np.dot(v.astype(np.float64), v)) - 1.0) < 1e-6  # stored unit-normalised
    small = np.load(GOLD / "small_data.npz")
    raw = small["labels"][0].astype(np.float64)
    np.testing.assert_allclose(v, raw / np.linalg.norm(raw), rtol=1e-6)
    # memory_usage = count*(pd*4 + (1+2M)*4 + 16 + 2) + upper_used*4 (index.cpp:365-371)
    pd, M0 = 16, 12
    assert ix.memory_usage >= 300 * (pd * 4 + (1 + M0) * 4 + 18)
    ix.mark_deleted(1000)
    ix.mark_deleted(1000)  # idempotent
    assert ix.is_deleted(1000)
    with pytest.raises(ValueError, match="unknown label"):
        ix.mark_deleted(999999)
    with pytest.raises(ValueError):
        ix.get_vector(1001)
    m = hg.Index.load(GOLD / "labels.idx", mmap=True)
    assert m.read_only
    with pytest.raises(RuntimeError, match="read-only"):
        m.add(np.zeros((1, 6), dtype=np.float32), ids=[5])
    m.mark_deleted(1006)  # tombstones live in memory: allowed on a mapped index
    assert m.is_deleted(1006)
    m.set_ef(77)
    assert m.ef == 77


def test_invalid_arguments(hg):
    with pytest.raises(ValueError):
        hg.Index(0)
    with pytest.raises(ValueError):
        hg.Index(4, M=1)
    with pytest.raises(ValueError):
        hg.Index(4, ef_construction=0)
    ix = hg.Index(4)
    with pytest.raises(ValueError):
        ix.set_ef(0)
    data = np.random.default_rng(1).uniform(-1, 1, size=(4, 4)).astype(np.float32)
    ix.add(data[:1], ids=[7])
    with pytest.raises(ValueError, match="already exists"):
        ix.add(data[1:2], ids=[7])
    with pytest.raises(ValueError, match="duplicate label"):
        ix.add(data[1:3], ids=[9, 9])
    with pytest.raises(ValueError):
        ix.add(data[1:3], ids=[10, 7])
    assert len(ix) == 1 and 10 not in ix  # failed batches insert nothing
    with pytest.raises(ValueError, match="k must be > 0"):
        ix.search_raw(data[:1], k=0)
    full = hg.Index(4, max_elements=2)
    full.add(data[:2])
    with pytest.raises(RuntimeError, match="full"):
        full.add(data[2:3], ids=[100])


def test_empty_index_needs_no_gpu(hg):
    ix = hg.Index(8)
    rec = ix.search_raw(np.zeros((2, 8), dtype=np.float32), k=3, ef=10)
    assert (rec["label"] == hg.INVALID_LABEL).all() and np.isinf(rec["distance"]).all()
    assert ix.search_one(np.zeros(8, dtype=np.float32), k=5).size == 0


def test_distance_order_registry(hg):
    assert hg.distance_order() in ("avx512", "avx2", "neon", "scalar")
    prev = hg.distance_order()
    hg.set_distance_order("neon")
    assert hg.distance_order() == "neon"
    hg.set_distance_order(prev)
