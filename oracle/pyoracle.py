"""ctypes binding of the C oracle (liboracle.so) -- test infrastructure only.

Used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg to
check (never to produce) the GPU library's results.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "liboracle.so"

METRICS = {"l2": 0, "ip": 1, "cosine": 2}
ISAS = {"scalar": 0, "avx2": 1, "avx512": 2, "neon": 3}
CNT_N = 7  # per-query traversal counters, see hnsw_oracle.c
INVALID_LABEL = np.uint64(0xFFFFFFFFFFFFFFFF)


def build() -> Path:
    """Compile liboracle.so (cheap; re-run when the source is newer)."""
    src = HERE / "hnsw_oracle.c"
    if not LIB_PATH.exists() or LIB_PATH.stat().st_mtime < src.stat().st_mtime:
        subprocess.run(["make", "-s", "-C", str(HERE), "liboracle.so"], check=True)
    return LIB_PATH


class _Info(C.Structure):
    _fields_ = [("dim", C.c_uint64), ("pd", C.c_uint64), ("M", C.c_uint64), ("count", C.c_uint64),
                ("ef_search", C.c_uint64), ("num_deleted", C.c_uint64), ("metric", C.c_int64),
                ("max_level", C.c_int64), ("entry", C.c_int64)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB_PATH))
        L.orc_load.restype = C.c_void_p
        L.orc_load.argtypes = [C.c_char_p, C.c_char_p, C.c_size_t]
        L.orc_free.argtypes = [C.c_void_p]
        L.orc_info.argtypes = [C.c_void_p, C.POINTER(_Info)]
        L.orc_set_isa.argtypes = [C.c_void_p, C.c_int]
        L.orc_set_ef.argtypes = [C.c_void_p, C.c_uint64]
        L.orc_mark_deleted.argtypes = [C.c_void_p, C.c_uint64]
        L.orc_search_batch.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_size_t, C.c_size_t, C.c_void_p,
                                       C.c_void_p, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.c_void_p, C.c_size_t]
        L.orc_search.restype = C.c_long
        L.orc_search.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_size_t, C.c_void_p, C.c_uint64, C.c_int,
                                 C.c_void_p, C.c_void_p]
        L.orc_bruteforce.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_size_t, C.c_int, C.c_int, C.c_void_p,
                                     C.c_size_t, C.c_size_t, C.c_void_p, C.c_uint64, C.c_int, C.c_void_p, C.c_void_p,
                                     C.c_size_t]
        L.orc_distance.restype = C.c_float
        L.orc_distance.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_size_t]
        L.orc_kernel.restype = C.c_float
        L.orc_kernel.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_size_t]
        L.orc_prepare_vector.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_size_t]
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def host_isa() -> str:
    """The ISA the reference would pick on this host (AVX-512 on x86 with it, NEON on Arm)."""
    m = os.uname().machine
    if m in ("aarch64", "arm64"):
        return "neon"
    flags = ""
    try:
        flags = Path("/proc/cpuinfo").read_text()
    except OSError:
        pass
    if " avx512f" in flags:
        return "avx512"
    if " avx2" in flags and " fma" in flags:
        return "avx2"
    return "scalar"


class OracleError(RuntimeError):
    pass


class OracleIndex:
    """A loaded index file searched on the CPU exactly as the reference does."""

    def __init__(self, path, isa: str = "avx512"):
        err = C.create_string_buffer(512)
        h = lib().orc_load(str(path).encode(), err, 512)
        if not h:
            raise OracleError(err.value.decode())
        self._h = h
        self.set_isa(isa)
        info = _Info()
        lib().orc_info(h, C.byref(info))
        self.dim, self.pd, self.M, self.count = info.dim, info.pd, info.M, info.count
        self.ef_search, self.metric, self.max_level = info.ef_search, info.metric, info.max_level

    def __del__(self):
        if getattr(self, "_h", None):
            lib().orc_free(self._h)
            self._h = None

    def set_isa(self, isa: str):
        lib().orc_set_isa(self._h, ISAS[isa])

    def mark_deleted(self, label: int):
        if lib().orc_mark_deleted(self._h, int(label)) != 0:
            raise ValueError(f"unknown label {label}")

    def search_batch(self, queries, k, ef=0, ef_per_query=None, k_per_query=None, filters=None, fsel=None,
                     threads=0, counters=False):
        """Returns (labels uint64 [nq,k], dists float32 [nq,k][, counters uint64 [nq,CNT_N]])."""
        q = np.ascontiguousarray(queries, dtype=np.float32)
        nq = q.shape[0]
        labels = np.empty((nq, k), dtype=np.uint64)
        dists = np.empty((nq, k), dtype=np.float32)
        cnt = np.zeros((nq, CNT_N), dtype=np.uint64) if counters else None
        efq = None if ef_per_query is None else np.ascontiguousarray(ef_per_query, dtype=np.uint64)
        kq = None if k_per_query is None else np.ascontiguousarray(k_per_query, dtype=np.uint64)
        fw = fs = None
        nf = 0
        keep = []
        if filters:
            nf = len(filters)
            arrs = [np.ascontiguousarray(w, dtype=np.uint64) for (w, _) in filters]
            keep.extend(arrs)
            fw = (C.c_void_p * nf)(*[a.ctypes.data for a in arrs])
            fs = np.array([s for (_, s) in filters], dtype=np.uint64)
        fsel_a = None if fsel is None else np.ascontiguousarray(fsel, dtype=np.int32)
        rc = lib().orc_search_batch(self._h, _ptr(q), nq, k, ef, _ptr(efq), _ptr(kq),
                                    C.cast(fw, C.c_void_p) if fw is not None else None, _ptr(fs), nf,
                                    _ptr(fsel_a), _ptr(labels), _ptr(dists), _ptr(cnt), threads)
        if rc != 0:
            raise ValueError("search_batch: k must be > 0")
        return (labels, dists, cnt) if counters else (labels, dists)

    def search(self, q, k, ef=0, filt=None):
        q = np.ascontiguousarray(q, dtype=np.float32)
        labels = np.empty(k, dtype=np.uint64)
        dists = np.empty(k, dtype=np.float32)
        if filt is None:
            m = lib().orc_search(self._h, _ptr(q), k, ef, None, 0, 0, _ptr(labels), _ptr(dists))
        else:
            w = np.ascontiguousarray(filt[0], dtype=np.uint64)
            m = lib().orc_search(self._h, _ptr(q), k, ef, _ptr(w), int(filt[1]), 1, _ptr(labels), _ptr(dists))
        if m < 0:
            raise ValueError("search: k must be > 0")
        return labels[:m], dists[:m]


def bruteforce(data, queries, k, metric="l2", isa="avx512", labels=None, filt=None, threads=0):
    d = np.ascontiguousarray(data, dtype=np.float32)
    q = np.ascontiguousarray(queries, dtype=np.float32)
    n, dim = d.shape
    nq = q.shape[0]
    out_l = np.empty((nq, k), dtype=np.uint64)
    out_d = np.empty((nq, k), dtype=np.float32)
    lab = None if labels is None else np.ascontiguousarray(labels, dtype=np.uint64)
    if filt is None:
        fw, fsz, has = None, 0, 0
    else:
        fw, fsz, has = np.ascontiguousarray(filt[0], dtype=np.uint64), int(filt[1]), 1
    rc = lib().orc_bruteforce(_ptr(d), _ptr(lab), n, dim, METRICS[metric], ISAS[isa], _ptr(q), nq, k, _ptr(fw), fsz,
                              has, _ptr(out_l), _ptr(out_d), threads)
    if rc != 0:
        raise ValueError("bruteforce: k must be > 0")
    return out_l, out_d


def kernel(isa: str, l2: bool, a, b) -> np.float32:
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = np.ascontiguousarray(b, dtype=np.float32)
    return np.float32(lib().orc_kernel(ISAS[isa], 1 if l2 else 0, _ptr(a), _ptr(b), a.shape[0]))


def prepare_vector(metric: str, v):
    v = np.ascontiguousarray(v, dtype=np.float32)
    out = np.empty_like(v)
    lib().orc_prepare_vector(METRICS[metric], _ptr(v), _ptr(out), v.shape[0])
    return out
