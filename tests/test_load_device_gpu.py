"""Index.load(path, device=N): the graph built on the device while the file is
read (FORMAT v1 sections 0-2 streamed through pinned staging buffers, layer 0
laid out on the device) must answer exactly like Index.load followed by the
usual upload, reject every file Index.load rejects with the same message, and
leave a host index that saves the same bytes."""
from __future__ import annotations

import hashlib
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = Path(__file__).resolve().parent / "golden"


def _same(a, b):
    np.testing.assert_array_equal(a["label"], b["label"])
    assert a["distance"].tobytes() == b["distance"].tobytes()


@pytest.mark.parametrize("name,deleted", [("c1", False), ("c3s", True)])
def test_streamed_load_answers_like_load(hg, graphs, tmp_path, name, deleted):
    path = graphs.path(name, deleted)
    _, q, *_ = graphs.data(name)
    ref = hg.Index.load(path)
    want = ref.search_raw(q, 10, 64)
    want16 = ref.search_batch_ex(q, 10, 64, precision=1, lists_per_step=2)
    src = hashlib.sha256(Path(path).read_bytes()).hexdigest()
    for mmap in (False, True):
        ix = hg.Index.load(path, mmap, device=0)
        assert ix.read_only == mmap
        _same(ix.search_raw(q, 10, 64), want)
        _same(ix.search_batch_ex(q, 10, 64, precision=1, lists_per_step=2), want16)
        out = tmp_path / f"{name}_{int(mmap)}.idx"
        ix.save(out)
        assert hashlib.sha256(out.read_bytes()).hexdigest() == src


def test_streamed_load_spans_several_staging_buffers(hg, tmp_path):
    """Sections larger than one 32 MiB staging buffer (70,000 x 128 floats)."""
    r = np.random.default_rng(9)
    base = r.normal(size=(70_000, 128)).astype(np.float32)
    q = r.normal(size=(300, 128)).astype(np.float32)
    ix0 = hg.Index(128, "l2", 8, 32)
    ix0.add(base)
    for lab in range(0, 70_000, 97):
        ix0.mark_deleted(lab)
    path = tmp_path / "big.idx"
    ix0.save(path)
    want = hg.Index.load(path).search_raw(q, 10, 48)
    for mmap in (False, True):
        _same(hg.Index.load(path, mmap, device=0).search_raw(q, 10, 48), want)


def test_streamed_load_rejects_what_load_rejects(hg, golden, tmp_path):
    meta, _ = golden
    fz = meta["fuzz"]
    src = (GOLD / fz["file"]).read_bytes()
    bad = tmp_path / "bad.idx"

    def message(fn):
        with pytest.raises(RuntimeError) as e:
            fn()
        return str(e.value)

    cases = []
    for pos, bit in fz["flips"]:
        b = bytearray(src)
        b[pos] ^= 1 << bit
        cases.append(bytes(b))
    cases += [src[:c] for c in fz["cuts"]]
    cases.append(src + b"\0")
    for data in cases:
        bad.write_bytes(data)
        for mmap in (False, True):
            if mmap and data == src + b"\0":
                continue
            want = message(lambda: hg.Index.load(bad, mmap))
            got = message(lambda: hg.Index.load(bad, mmap, device=0))
            assert got == want
    for mmap in (False, True):
        with pytest.raises(RuntimeError):
            hg.Index.load(tmp_path / "missing.idx", mmap, device=0)
