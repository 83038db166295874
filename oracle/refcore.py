"""ctypes binding of the reference hnsw-engine library (oracle/_ref/libhnswref.so).

Test and benchmark infrastructure only.  The library is the reference's own
C++ code compiled from its sources by oracle/Makefile (``make -C oracle
ref-if-present``), on this machine's architecture: NEON kernels on aarch64,
AVX2 / AVX-512 on x86-64, as the reference selects at run time.  It serves
three purposes:

* graphs: ``build`` runs the reference's ``Index::add_batch``
  (src/index.cpp:273-306) and ``save`` (src/persist.cpp) -- the graph files
  the GPU library loads;
* the CPU baseline: ``RefIndex.search_batch`` times the reference's own
  ``Index::search_batch`` (src/search_layer.cpp:180-194) on the host cores;
* parity: its ids and distances are what the GPU path must reproduce.

Nothing in the GPU library imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_ref" / "libhnswref.so"
NEIGHBOR = np.dtype([("label", "<u8"), ("distance", "<f4"), ("pad", "<u4")])

_lib = None


class RefUnavailable(RuntimeError):
    """The reference library could not be built or loaded on this machine."""


def available() -> bool:
    try:
        lib()
        return True
    except RefUnavailable:
        return False


def lib():
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        r = subprocess.run(["make", "-s", "-C", str(HERE), "ref-if-present"], capture_output=True, text=True)
        if not LIB_PATH.exists():
            raise RefUnavailable("reference library not built: " + (r.stdout + r.stderr).strip()[-300:])
    L = C.CDLL(str(LIB_PATH))
    sz, vp, cp = C.c_size_t, C.c_void_p, C.c_char_p
    L.ref_isa.argtypes = [C.c_char_p, sz]
    L.ref_build.argtypes = [vp, vp, sz, sz, cp, sz, sz, C.c_uint64, sz, cp, cp, sz]
    L.ref_load.argtypes = [cp, C.c_int, C.POINTER(vp), cp, sz]
    L.ref_free.argtypes = [vp]
    L.ref_info.argtypes = [vp, vp]
    L.ref_mark_deleted.argtypes = [vp, C.c_uint64, cp, sz]
    L.ref_set_ef.argtypes = [vp, sz, cp, sz]
    L.ref_save.argtypes = [vp, cp, cp, sz]
    L.ref_filter_new.restype = vp
    L.ref_filter_new.argtypes = [vp, C.c_uint64]
    L.ref_filter_free.argtypes = [vp]
    L.ref_search_batch.argtypes = [vp, vp, sz, sz, sz, vp, sz, vp, cp, sz]
    L.ref_search.argtypes = [vp, vp, sz, sz, vp, vp, C.POINTER(sz), cp, sz]
    L.ref_bruteforce.argtypes = [vp, vp, sz, sz, cp, vp, sz, sz, vp, sz, vp, cp, sz]
    L.ref_kernels.argtypes = [cp, vp, vp, sz, sz, vp, cp, sz]
    _lib = L
    return L


def _call(fn, *args):
    err = C.create_string_buffer(512)
    if fn(*args, err, 512) != 0:
        msg = err.value.decode(errors="replace")
        raise (ValueError if "invalid" in msg or "unknown" in msg else RuntimeError)(msg)


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def isa() -> str:
    buf = C.create_string_buffer(32)
    lib().ref_isa(buf, 32)
    return buf.value.decode()


def build(vectors, path, metric: str = "l2", M: int = 16, ef_construction: int = 200, seed: int = 100,
          threads: int = 0, labels=None) -> Path:
    """The reference's add_batch over `vectors` (labels 0..n-1 unless given),
    saved to `path` in its file format.  threads = 0: all host threads (the
    graph then depends on thread timing); 1: deterministic."""
    v = np.ascontiguousarray(vectors, dtype=np.float32)
    lab = None if labels is None else np.ascontiguousarray(labels, dtype=np.uint64)
    _call(lib().ref_build, _p(v), _p(lab), v.shape[0], v.shape[1], metric.encode(), M, ef_construction, seed,
          threads, str(path).encode())
    return Path(path)


def kernels(isa_name: str, a, b):
    """(l2_sq, dot) of each row pair under the named ISA's kernels."""
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = np.ascontiguousarray(b, dtype=np.float32)
    out = np.empty((a.shape[0], 2), dtype=np.float32)
    _call(lib().ref_kernels, isa_name.encode(), _p(a), _p(b), a.shape[1], a.shape[0], _p(out))
    return out[:, 0], out[:, 1]


class Bitset:
    """A reference BitsetFilter over labels [0, bits) from u64 words."""

    def __init__(self, words, bits: int):
        self.words = np.ascontiguousarray(words, dtype=np.uint64)
        self.h = lib().ref_filter_new(_p(self.words), int(bits))

    def __del__(self):
        if getattr(self, "h", None):
            lib().ref_filter_free(self.h)
            self.h = None


def bruteforce(vectors, queries, k: int, metric: str = "l2", threads: int = 0, filt: Bitset | None = None):
    v = np.ascontiguousarray(vectors, dtype=np.float32)
    q = np.ascontiguousarray(queries, dtype=np.float32)
    out = np.empty(q.shape[0] * k, dtype=NEIGHBOR)
    _call(lib().ref_bruteforce, _p(v), None, v.shape[0], v.shape[1], metric.encode(), _p(q), q.shape[0], k, _p(out),
          threads, filt.h if filt else None)
    return out.reshape(q.shape[0], k)


class RefIndex:
    """A graph file loaded by the reference's Index::load."""

    def __init__(self, path, mmap: bool = False):
        h = C.c_void_p()
        _call(lib().ref_load, str(path).encode(), int(mmap), C.byref(h))
        self.h = h
        info = np.zeros(4, dtype=np.uint64)
        lib().ref_info(self.h, _p(info))
        self.size, self.dim, self.ef, self.max_level = (int(x) for x in info)

    def __del__(self):
        if getattr(self, "h", None):
            lib().ref_free(self.h)
            self.h = None

    def mark_deleted(self, label: int):
        _call(lib().ref_mark_deleted, self.h, int(label))

    def set_ef(self, ef: int):
        _call(lib().ref_set_ef, self.h, int(ef))

    def save(self, path):
        _call(lib().ref_save, self.h, str(path).encode())

    def search_batch(self, queries, k: int, ef: int = 0, threads: int = 0, filt: Bitset | None = None, out=None):
        q = np.ascontiguousarray(queries, dtype=np.float32)
        if out is None:
            out = np.empty(q.shape[0] * k, dtype=NEIGHBOR)
        _call(lib().ref_search_batch, self.h, _p(q), q.shape[0], k, ef, _p(out), threads, filt.h if filt else None)
        return out.reshape(q.shape[0], k)

    def search(self, query, k: int, ef: int = 0, filt: Bitset | None = None):
        q = np.ascontiguousarray(query, dtype=np.float32)
        out = np.empty(max(k, 1), dtype=NEIGHBOR)
        n = C.c_size_t()
        _call(lib().ref_search, self.h, _p(q), k, ef, filt.h if filt else None, _p(out), C.byref(n))
        return out[: n.value]


def host_threads() -> int:
    return os.cpu_count() or 1
