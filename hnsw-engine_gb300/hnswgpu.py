"""Python binding of libhnswgpu over its C ABI (include/hnswgpu.h).

Mirrors the reference's Python module (python/bindings.cpp:114-233): the same
``Index`` constructor, ``add`` / ``search`` / ``save`` / ``load`` /
``mark_deleted`` / properties, the same filter forms (None, a callable on
labels, a bool mask over labels, an integer allow-list) and the same int64
ids with -1 padding.  Queries are answered on the GPU; there is no CPU search
path, and importing this module without the built library raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "lib" / "libhnswgpu.so"

HG_OK, HG_EINVAL, HG_ERUNTIME, HG_ERANGE = 0, 1, 2, 3
METRICS = {"l2": 0, "ip": 1, "inner_product": 1, "cosine": 2}
METRIC_NAMES = {0: "l2", 1: "ip", 2: "cosine"}
ORDERS = {"scalar": 0, "avx2": 1, "avx512": 2, "neon": 3}
INVALID_LABEL = 0xFFFFFFFFFFFFFFFF
NCOUNTERS = 8

NEIGHBOR = np.dtype([("label", "<u8"), ("distance", "<f4"), ("reserved", "<u4")])

PRED = C.CFUNCTYPE(C.c_int, C.c_uint64, C.c_void_p)


class _Filter(C.Structure):
    _fields_ = [("kind", C.c_int32), ("reserved", C.c_int32), ("words", C.c_void_p), ("num_labels", C.c_uint64),
                ("fn", PRED), ("ctx", C.c_void_p)]


class _BatchOptions(C.Structure):
    _fields_ = [("ef_per_query", C.c_void_p), ("k_per_query", C.c_void_p), ("filters", C.POINTER(_Filter)),
                ("num_filters", C.c_size_t), ("filter_of_query", C.c_void_p), ("stream", C.c_void_p),
                ("precision", C.c_int32), ("use_graph", C.c_int32), ("counters", C.c_void_p),
                ("hash_slots", C.c_uint32), ("cand_cap", C.c_uint32), ("warps_per_block", C.c_uint32),
                ("pool_cap", C.c_uint32), ("queries_on_device", C.c_int32), ("out_on_device", C.c_int32),
                ("filter_scan_permille", C.c_uint32), ("rerank_factor", C.c_uint32),
                ("warps_per_query", C.c_uint32), ("lists_per_step", C.c_uint32),
                ("filter_scan_mode", C.c_uint32), ("reserved", C.c_uint32)]


class _ServerConfig(C.Structure):
    _fields_ = [("max_inflight", C.c_uint32), ("max_batch_queries", C.c_uint32), ("memory_budget", C.c_uint64),
                ("precision", C.c_int32), ("filter_scan_permille", C.c_uint32), ("rerank_factor", C.c_uint32),
                ("warps_per_query", C.c_uint32), ("lists_per_step", C.c_uint32),
                ("filter_scan_mode", C.c_uint32)]


class _Request(C.Structure):
    _fields_ = [("queries", C.c_void_p), ("nq", C.c_uint32), ("k", C.c_uint32), ("ef", C.c_uint32),
                ("reserved", C.c_uint32), ("filter", C.POINTER(_Filter)), ("out", C.c_void_p)]


class _BuildOptions(C.Structure):
    _fields_ = [("device", C.c_int32), ("wave_min", C.c_uint32), ("wave_max", C.c_uint32), ("waves", C.c_uint32),
                ("wave_fraction", C.c_double), ("dropped_proposals", C.c_uint64), ("seconds", C.c_double),
                ("peers", C.c_int32), ("reserved", C.c_int32)]


class _ServerStats(C.Structure):
    _fields_ = [("requests", C.c_uint64), ("queries", C.c_uint64), ("batches", C.c_uint64),
                ("memory_waits", C.c_uint64), ("elapsed_s", C.c_double), ("qps", C.c_double),
                ("p50_ms", C.c_double), ("p99_ms", C.c_double), ("p999_ms", C.c_double), ("mean_ms", C.c_double),
                ("max_ms", C.c_double), ("mean_batch_queries", C.c_double)]


_lib = None


def lib():
    """The loaded libhnswgpu.so; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: run __graft_entry__.build() (or hnsw-engine_gb300/build.py)")
        L = C.CDLL(str(LIB_PATH))
        vp, sz, u64, i32 = C.c_void_p, C.c_size_t, C.c_uint64, C.c_int
        L.hg_last_error.restype = C.c_char_p
        L.hg_index_create.argtypes = [sz, i32, sz, sz, sz, u64, C.POINTER(vp)]
        L.hg_index_load.argtypes = [C.c_char_p, i32, C.POINTER(vp)]
        L.hg_index_load_device.argtypes = [C.c_char_p, i32, i32, C.POINTER(vp)]
        L.hg_index_save.argtypes = [vp, C.c_char_p]
        L.hg_index_free.argtypes = [vp]
        L.hg_index_add_batch.argtypes = [vp, vp, vp, sz, sz]
        L.hg_index_add_batch_gpu.argtypes = [vp, vp, vp, sz, C.POINTER(_BuildOptions)]
        L.hg_index_search.argtypes = [vp, vp, sz, sz, C.POINTER(_Filter), vp, C.POINTER(sz)]
        L.hg_index_search_batch.argtypes = [vp, vp, sz, sz, sz, vp, sz, C.POINTER(_Filter)]
        L.hg_index_search_batch_ex.argtypes = [vp, vp, sz, sz, sz, vp, C.POINTER(_BatchOptions)]
        L.hg_index_mark_deleted.argtypes = [vp, u64]
        L.hg_index_is_deleted.argtypes = [vp, u64, C.POINTER(i32)]
        L.hg_index_contains.argtypes = [vp, u64, C.POINTER(i32)]
        L.hg_index_get_vector.argtypes = [vp, u64, vp, sz]
        L.hg_index_set_ef.argtypes = [vp, sz]
        L.hg_index_set_device.argtypes = [vp, i32]
        for name in ("size", "dim", "M", "ef_construction", "ef", "capacity", "memory_usage"):
            fn = getattr(L, f"hg_index_{name}")
            fn.argtypes = [vp]
            fn.restype = sz
        for name in ("metric", "max_level", "read_only"):
            fn = getattr(L, f"hg_index_{name}")
            fn.argtypes = [vp]
            fn.restype = i32
        L.hg_bruteforce_create.argtypes = [sz, i32, C.POINTER(vp)]
        L.hg_bruteforce_add.argtypes = [vp, vp, vp, sz]
        L.hg_bruteforce_search_batch.argtypes = [vp, vp, sz, sz, vp, C.POINTER(_Filter)]
        L.hg_bruteforce_free.argtypes = [vp]
        L.hg_index_search_batch_noalloc.argtypes = [vp, vp, sz, sz, sz, vp, vp]
        L.hg_index_autotune.argtypes = [vp, vp, sz, sz, sz, i32, vp, C.c_char_p, sz, C.POINTER(sz)]
        L.hg_index_set_tuning.argtypes = [vp, C.c_char_p]
        L.hg_bruteforce_set_path.argtypes = [vp, i32]
        L.hg_bruteforce_last_path.argtypes = [vp]
        L.hg_server_create.argtypes = [vp, C.POINTER(_ServerConfig), C.POINTER(vp)]
        L.hg_server_submit.argtypes = [vp, C.POINTER(_Request), C.POINTER(C.c_uint64)]
        L.hg_server_wait.argtypes = [vp, C.c_uint64, C.POINTER(C.c_double)]
        L.hg_server_replay.argtypes = [vp, C.POINTER(_Request), vp, sz, C.POINTER(_ServerStats)]
        L.hg_server_replay_latencies.argtypes = [vp, C.POINTER(_Request), vp, sz, C.POINTER(_ServerStats), vp]
        L.hg_server_stats_get.argtypes = [vp, C.POINTER(_ServerStats)]
        L.hg_server_destroy.argtypes = [vp]
        L.hg_set_distance_order.argtypes = [i32]
        L.hg_get_distance_order.restype = i32
        _lib = L
    return _lib


def _check(rc: int):
    if rc == HG_OK:
        return
    msg = lib().hg_last_error().decode(errors="replace")
    if rc == HG_EINVAL:
        raise ValueError(msg)
    if rc == HG_ERANGE:
        raise IndexError(msg)
    raise RuntimeError(msg)


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def set_distance_order(name: str):
    """Summation order reproduced by indexes created/loaded afterwards (simd::set_active)."""
    _check(lib().hg_set_distance_order(ORDERS[name]))


def distance_order() -> str:
    return {v: k for k, v in ORDERS.items()}[lib().hg_get_distance_order()]


def simd_isa() -> str:
    """The host kernel order in use (the reference's simd_isa())."""
    return distance_order()


def _rerank_factor(v) -> int:
    v = int(v)
    if v < 0:
        raise ValueError("rerank_factor must be >= 0 (0 reranks the whole pool)")
    return v


def _warps_per_query(v) -> int:
    v = int(v)
    if v not in (0, 1, 4):
        raise ValueError("warps_per_query must be 1 (one warp, the reference's order) or 4 (beam search)")
    return v


def _lists_per_step(v) -> int:
    v = int(v)
    if not 0 <= v <= 4:
        raise ValueError("lists_per_step must be 0 (the reference's order) or 1..4 (beam search)")
    return v


SCAN_MODES = {"auto": 0, "allowed_rows": 1, "every_row": 2}


def _scan_mode(v) -> int:
    if v not in SCAN_MODES:
        raise ValueError("filter_scan_mode must be 'auto', 'allowed_rows' or 'every_row'")
    return SCAN_MODES[v]


def _float_matrix(x, name: str) -> np.ndarray:
    """float32, C-contiguous; non-numeric input is a TypeError (as in the reference's binding)."""
    arr = np.asarray(x)
    if arr.dtype.kind not in "biuf":
        raise TypeError(f"{name}: expected a numeric array, got dtype {arr.dtype}")
    return np.ascontiguousarray(arr, dtype=np.float32)


def _to_labels(ids, n: int, start: int) -> np.ndarray:
    if ids is None:
        return np.arange(start, start + n, dtype=np.uint64)
    arr = np.asarray(ids)
    if arr.ndim == 0:
        arr = arr.reshape(1)
    if arr.ndim != 1 or arr.shape[0] != n:
        raise ValueError(f"ids: expected shape ({n},)")
    if arr.dtype.kind == "i":
        if (arr < 0).any():
            raise ValueError("ids: labels must be non-negative")
        return arr.astype(np.uint64)
    if arr.dtype.kind == "u":
        return arr.astype(np.uint64)
    raise TypeError("ids: expected an integer array")


class _FilterHolder:
    """Keeps a C filter description and the memory it points to alive."""

    def __init__(self, spec):
        self.struct = None
        self.keep = []
        self.error = None  # an exception raised by a callable filter
        if spec is None:
            return
        f = _Filter()
        if isinstance(spec, (np.ndarray, list, tuple)):
            arr = np.asarray(spec)
            if arr.ndim != 1:
                raise ValueError("filter: expected a 1-D array")
            if arr.dtype.kind == "b":
                words = _pack_mask(arr)
                f.kind, f.num_labels = 1, arr.shape[0]
            elif arr.dtype.kind in "iu":
                labels = _to_labels(arr, arr.shape[0], 0)
                size = int(labels.max()) + 1 if labels.size else 0
                mask = np.zeros(size, dtype=bool)
                mask[labels.astype(np.int64)] = True
                words = _pack_mask(mask)
                f.kind, f.num_labels = 1, size
            else:
                raise TypeError("filter: array must be bool (mask over labels) or integer (allowed labels)")
            self.keep.append(words)
            f.words = words.ctypes.data
        elif isinstance(spec, tuple) is False and hasattr(spec, "words") and hasattr(spec, "num_labels"):
            words = np.ascontiguousarray(spec.words, dtype=np.uint64)
            self.keep.append(words)
            f.kind, f.words, f.num_labels = 1, words.ctypes.data, int(spec.num_labels)
        elif callable(spec):
            def call(label, ctx):
                if self.error is not None:
                    return 0
                try:
                    return 1 if spec(int(label)) else 0
                except BaseException as e:  # re-raised by raise_pending() after the call
                    self.error = e
                    return 0

            fn = PRED(call)
            self.keep.append(fn)
            f.kind, f.fn = 2, fn
        else:
            raise TypeError("filter: expected None, a callable(label) -> bool, a bool mask or an id array")
        self.struct = f

    def ref(self):
        return None if self.struct is None else C.byref(self.struct)

    def raise_pending(self):
        if self.error is not None:
            raise self.error


def _pack_mask(mask: np.ndarray) -> np.ndarray:
    n = mask.shape[0]
    nwords = max((n + 63) // 64, 1)
    padded = np.zeros(nwords * 64, dtype=bool)
    padded[:n] = mask
    return np.packbits(padded.reshape(-1, 8), axis=1, bitorder="little").reshape(-1).view(np.uint64).copy()


class Bitset:
    """A BitsetFilter given directly as words (bit l of words[l >> 6])."""

    def __init__(self, words, num_labels: int):
        self.words = np.ascontiguousarray(words, dtype=np.uint64)
        self.num_labels = int(num_labels)


class Index:
    """HNSW index (hnsw::Index); construction on the CPU, queries on the GPU."""

    def __init__(self, dim: int = 0, metric: str = "l2", M: int = 16, ef_construction: int = 200,
                 max_elements: int = 0, seed: int = 100, _handle=None):
        self._h = None
        if _handle is not None:
            self._h = _handle
            return
        h = C.c_void_p()
        if metric not in METRICS:
            raise ValueError(f"unknown metric '{metric}' (expected l2, ip or cosine)")
        _check(lib().hg_index_create(dim, METRICS[metric], M, ef_construction, max_elements, seed, C.byref(h)))
        self._h = h

    def __del__(self):
        if getattr(self, "_h", None):
            lib().hg_index_free(self._h)
            self._h = None

    @staticmethod
    def load(path, mmap: bool = False, device=None) -> "Index":
        """Index::load.  device=N also builds the graph on CUDA device N in the
        same pass (the file's sections streamed through pinned staging
        buffers while they are read and hashed)."""
        h = C.c_void_p()
        if device is None:
            _check(lib().hg_index_load(str(path).encode(), 1 if mmap else 0, C.byref(h)))
        else:
            _check(lib().hg_index_load_device(str(path).encode(), 1 if mmap else 0, int(device), C.byref(h)))
        return Index(_handle=h)

    def save(self, path):
        _check(lib().hg_index_save(self._h, str(path).encode()))

    def add(self, vectors, ids=None, num_threads: int = 0):
        v = _float_matrix(vectors, "vectors")
        if v.ndim == 1:
            v = v.reshape(1, -1)
        if v.shape[1] != self.dim:
            raise ValueError(f"vectors: expected shape (n, {self.dim})")
        labels = _to_labels(ids, v.shape[0], len(self))
        _check(lib().hg_index_add_batch(self._h, _ptr(v), _ptr(labels), v.shape[0], num_threads))

    def add_gpu(self, vectors, ids=None, device: int = -1, wave_fraction: float = 0.0, wave_min: int = 0,
                wave_max: int = 0, peers: bool = False) -> dict:
        """add with the graph linking on the GPU (no counterpart in the
        reference): same validation, stored rows, labels and levels as add;
        the graph is judged on recall, not identity.  Returns the waves
        launched, the reverse edges dropped and the linking's wall time."""
        v = _float_matrix(vectors, "vectors")
        if v.ndim == 1:
            v = v.reshape(1, -1)
        if v.shape[1] != self.dim:
            raise ValueError(f"vectors: expected shape (n, {self.dim})")
        labels = _to_labels(ids, v.shape[0], len(self))
        o = _BuildOptions(device=int(device), wave_min=int(wave_min), wave_max=int(wave_max),
                          wave_fraction=float(wave_fraction), peers=1 if peers else 0)
        _check(lib().hg_index_add_batch_gpu(self._h, _ptr(v), _ptr(labels), v.shape[0], C.byref(o)))
        return {"waves": int(o.waves), "dropped_proposals": int(o.dropped_proposals), "seconds": float(o.seconds)}

    def _queries(self, queries):
        q = _float_matrix(queries, "queries")
        single = q.ndim == 1
        if single:
            q = q.reshape(1, -1)
        if q.ndim != 2 or q.shape[1] != self.dim:
            raise ValueError(f"queries: expected shape (n, {self.dim})")
        return q, single

    def search_raw(self, queries, k: int = 10, ef: int = 0, filter=None) -> np.ndarray:
        """search_batch into hnsw::Neighbor records (labels uint64, kInvalidLabel padding)."""
        if k <= 0:
            raise ValueError("k must be > 0")
        q, _ = self._queries(queries)
        out = np.empty(q.shape[0] * k, dtype=NEIGHBOR)
        fh = _FilterHolder(filter)
        rc = lib().hg_index_search_batch(self._h, _ptr(q), q.shape[0], k, ef or 0, _ptr(out), 0, fh.ref())
        fh.raise_pending()
        _check(rc)
        return out.reshape(q.shape[0], k)

    def search(self, queries, k: int = 10, ef=None, num_threads: int = 0, filter=None):
        """(ids int64 with -1 padding, distances float32), as the reference's binding returns."""
        if k <= 0:
            raise ValueError("k must be > 0")
        q, single = self._queries(queries)
        rec = self.search_raw(q, k, ef or 0, filter)
        ids = rec["label"].astype(np.int64)  # kInvalidLabel -> -1
        d = rec["distance"].copy()
        return (ids[0], d[0]) if single else (ids, d)

    def search_one(self, q, k: int = 10, ef: int = 0, filter=None):
        """Index::search: at most k results, no padding."""
        q = np.ascontiguousarray(q, dtype=np.float32).reshape(-1)
        out = np.empty(k, dtype=NEIGHBOR)
        n = C.c_size_t()
        fh = _FilterHolder(filter)
        rc = lib().hg_index_search(self._h, _ptr(q), k, ef, fh.ref(), _ptr(out), C.byref(n))
        fh.raise_pending()
        _check(rc)
        return out[:n.value]

    def search_batch_ex(self, queries, k: int, ef: int = 0, ef_per_query=None, k_per_query=None, filters=None,
                        filter_of_query=None, stream=None, precision: int = 0, counters: bool = False,
                        hash_slots: int = 0, cand_cap: int = 0, warps_per_block: int = 0, pool_cap: int = 0,
                        out=None, filter_scan: float = 0.0, rerank_factor: int = 0, warps_per_query: int = 1,
                        lists_per_step: int = 0, filter_scan_mode: str = "auto"):
        """search_batch with per-query ef / k / filter.  filter_scan (FP16 / FP8
        only): queries whose filter allows at most this fraction of the nodes
        are answered by an exact tensor-core scan instead of a graph walk;
        filter_scan_mode picks it: 'allowed_rows' (only the rows the filter
        allows), 'every_row' (the GEMM over all rows) or 'auto' (fewer bytes).
        rerank_factor (FP16 / FP8 only): the exact FP32 rerank covers the best
        rerank_factor x k entries of the traversal pool (at least 32); 0 = all.
        warps_per_query=4 (FP16 / FP8, dim <= 128): four warps walk each query
        as a beam search (lower latency per query; not the reference's visit
        order, so recall is the bar).  lists_per_step=1..4 (FP16 / FP8, dim <=
        128): one warp walks each query as a beam search expanding that many
        neighbour lists per step, row distances on the tensor cores (the
        throughput form; recall is the bar)."""
        q, _ = self._queries(queries)
        nq = q.shape[0]
        if out is None:
            out = np.empty(nq * k, dtype=NEIGHBOR)
        elif out.dtype != NEIGHBOR or out.size != nq * k or not out.flags.c_contiguous:
            raise ValueError("out: expected a contiguous NEIGHBOR array of nq*k records")
        opt = _BatchOptions()
        opt.filter_scan_permille = int(round(filter_scan * 1000))
        opt.rerank_factor = _rerank_factor(rerank_factor)
        opt.warps_per_query = _warps_per_query(warps_per_query)
        opt.lists_per_step = _lists_per_step(lists_per_step)
        opt.filter_scan_mode = _scan_mode(filter_scan_mode)
        keep = []
        if ef_per_query is not None:
            a = np.ascontiguousarray(ef_per_query, dtype=np.uint32)
            keep.append(a)
            opt.ef_per_query = a.ctypes.data
        if k_per_query is not None:
            a = np.ascontiguousarray(k_per_query, dtype=np.uint32)
            keep.append(a)
            opt.k_per_query = a.ctypes.data
        holders = [_FilterHolder(f) for f in (filters or [])]
        if holders:
            arr = (_Filter * len(holders))(*[h.struct for h in holders])
            keep.append(arr)
            opt.filters = C.cast(arr, C.POINTER(_Filter))
            opt.num_filters = len(holders)
        if filter_of_query is not None:
            a = np.ascontiguousarray(filter_of_query, dtype=np.int32)
            keep.append(a)
            opt.filter_of_query = a.ctypes.data
        if stream is not None:
            opt.stream = stream
        opt.precision = precision
        opt.hash_slots, opt.cand_cap = hash_slots, cand_cap
        opt.warps_per_block, opt.pool_cap = warps_per_block, pool_cap
        cnt = None
        if counters:
            cnt = np.zeros((nq, NCOUNTERS), dtype=np.uint64)
            opt.counters = cnt.ctypes.data
        rc = lib().hg_index_search_batch_ex(self._h, _ptr(q), nq, k, ef, _ptr(out), C.byref(opt))
        for h in holders:
            h.raise_pending()
        _check(rc)
        out = out.reshape(nq, k)
        return (out, cnt) if counters else out

    def search_device(self, q_ptr: int, nq: int, k: int, ef: int, out_ptr: int, stream: int = 0,
                      ef_ptr: int = 0, k_ptr: int = 0, graph: bool = False, precision: int = 0,
                      rerank_factor: int = 0, warps_per_query: int = 1, lists_per_step: int = 0):
        """Enqueue a batch whose queries (nq x dim float32), optional per-query
        ef / k (uint32) and output records (nq x k x 16 bytes) live in device
        memory; returns once the work is on `stream` (a cudaStream_t handle).
        graph=True: the launch sequence is captured into a CUDA graph on the
        second call with the same pointers and shape and replayed after."""
        opt = _BatchOptions()
        opt.queries_on_device, opt.out_on_device = 1, 1
        opt.use_graph = 1 if graph else 0
        opt.precision = precision
        opt.rerank_factor = _rerank_factor(rerank_factor)
        opt.warps_per_query = _warps_per_query(warps_per_query)
        opt.lists_per_step = _lists_per_step(lists_per_step)
        opt.ef_per_query = ef_ptr or None
        opt.k_per_query = k_ptr or None
        opt.stream = stream or None
        _check(lib().hg_index_search_batch_ex(self._h, C.c_void_p(q_ptr), nq, k, ef, C.c_void_p(out_ptr),
                                              C.byref(opt)))

    def autotune(self, queries, k: int = 10, ef_max: int = 512, precision: int = 0, path=None,
                 ef_per_query=None) -> dict:
        """Time the query kernel's launch shapes per ef bucket on these sample
        queries, install the fastest and return the table (also written to
        `path` as JSON when given).  With ef_per_query the sample runs as one
        mixed batch and the shapes are chosen on its total time."""
        import json

        q, _ = self._queries(queries)
        efq = None if ef_per_query is None else np.ascontiguousarray(ef_per_query, dtype=np.uint32)
        need = C.c_size_t(0)
        buf = C.create_string_buffer(1 << 16)
        _check(lib().hg_index_autotune(self._h, _ptr(q), q.shape[0], k, ef_max, precision, _ptr(efq), buf, len(buf),
                                       C.byref(need)))
        text = buf.value.decode()
        if path is not None:
            Path(path).write_text(text)
        return json.loads(text)

    def set_tuning(self, table):
        """Install a table from autotune (a dict, a JSON string or a file path)."""
        import json

        if isinstance(table, dict):
            text = json.dumps(table)
        elif isinstance(table, (str, Path)) and Path(str(table)).exists():
            text = Path(str(table)).read_text()
        else:
            text = str(table)
        _check(lib().hg_index_set_tuning(self._h, text.encode()))

    def search_noalloc(self, q_ptr: int, nq: int, k: int, ef: int, out_ptr: int, stream: int = 0):
        """hg_index_search_batch_noalloc: a batch that allocates no device memory.

        For callers that cannot call cudaMalloc while searching.  q_ptr (nq x dim
        float32) and out_ptr (nq x k 16-byte records) are device addresses the
        caller owns; scratch is the library's static device array, so batches
        overlapping on the GPU race.  The graph must already be on the GPU (run
        any allocating search once first).  Limits: nq <= 65536, index size
        <= 2^20, max(ef, k) <= 512."""
        _check(lib().hg_index_search_batch_noalloc(self._h, C.c_void_p(q_ptr), nq, k, ef, C.c_void_p(out_ptr),
                                                   C.c_void_p(stream) if stream else None))

    def set_ef(self, ef: int):
        _check(lib().hg_index_set_ef(self._h, ef))

    def set_device(self, device: int):
        _check(lib().hg_index_set_device(self._h, device))

    def mark_deleted(self, label: int):
        if label < 0:
            raise ValueError("labels are non-negative")
        _check(lib().hg_index_mark_deleted(self._h, int(label)))

    def is_deleted(self, label: int) -> bool:
        if label < 0:
            return False
        r = C.c_int()
        _check(lib().hg_index_is_deleted(self._h, int(label), C.byref(r)))
        return bool(r.value)

    def __contains__(self, label) -> bool:
        if label < 0:
            return False
        r = C.c_int()
        _check(lib().hg_index_contains(self._h, int(label), C.byref(r)))
        return bool(r.value)

    def get_vector(self, label: int) -> np.ndarray:
        if label < 0:
            raise ValueError("labels are non-negative")
        out = np.empty(self.dim, dtype=np.float32)
        _check(lib().hg_index_get_vector(self._h, int(label), _ptr(out), self.dim))
        return out

    def __len__(self):
        return lib().hg_index_size(self._h)

    @property
    def dim(self):
        return lib().hg_index_dim(self._h)

    @property
    def metric(self):
        return METRIC_NAMES[lib().hg_index_metric(self._h)]

    @property
    def M(self):
        return lib().hg_index_M(self._h)

    @property
    def ef_construction(self):
        return lib().hg_index_ef_construction(self._h)

    @property
    def ef(self):
        return lib().hg_index_ef(self._h)

    @ef.setter
    def ef(self, v):
        self.set_ef(v)

    @property
    def capacity(self):
        return lib().hg_index_capacity(self._h)

    @property
    def max_level(self):
        return lib().hg_index_max_level(self._h)

    @property
    def read_only(self):
        return bool(lib().hg_index_read_only(self._h))

    @property
    def memory_usage(self):
        return lib().hg_index_memory_usage(self._h)

    def __repr__(self):
        return (f"<hnswgpu.Index dim={self.dim} metric={self.metric} M={self.M} size={len(self)}"
                + (" read_only" if self.read_only else "") + ">")


class BruteForceIndex:
    """Exact k-NN (hnsw::BruteForceIndex) on the GPU."""

    def __init__(self, dim: int, metric: str = "l2"):
        self._h = None
        h = C.c_void_p()
        _check(lib().hg_bruteforce_create(dim, METRICS[metric], C.byref(h)))
        self._h = h
        self.dim = dim

    def __del__(self):
        if getattr(self, "_h", None):
            lib().hg_bruteforce_free(self._h)
            self._h = None

    def add(self, vectors, labels=None):
        v = np.ascontiguousarray(vectors, dtype=np.float32).reshape(-1, self.dim)
        lab = None if labels is None else np.ascontiguousarray(labels, dtype=np.uint64)
        _check(lib().hg_bruteforce_add(self._h, _ptr(v), _ptr(lab), v.shape[0]))

    def search_raw(self, queries, k: int, filter=None) -> np.ndarray:
        q = np.ascontiguousarray(queries, dtype=np.float32).reshape(-1, self.dim)
        out = np.empty(q.shape[0] * k, dtype=NEIGHBOR)
        fh = _FilterHolder(filter)
        _check(lib().hg_bruteforce_search_batch(self._h, _ptr(q), q.shape[0], k, _ptr(out), fh.ref()))
        return out.reshape(q.shape[0], k)

    PATH_AUTO, PATH_SCAN, PATH_TENSOR = 0, 1, 2

    def set_path(self, path: int):
        """GPU kernel: 0 auto, 1 CUDA-core scan, 2 tensor-core GEMM + exact rerank."""
        _check(lib().hg_bruteforce_set_path(self._h, path))

    @property
    def last_path(self) -> int:
        return int(lib().hg_bruteforce_last_path(self._h))


class Server:
    """Continuous-batching server over an Index (hg_server_*): requests with their
    own k / ef / filter are admitted into GPU batches as slots and memory free up.

    precision 1 / 2 serves with FP16 / FP8 traversal and an exact FP32 rerank;
    with those, filter_scan answers requests whose filter allows at most that
    fraction of the nodes by the exact tensor-core scan, rerank_factor limits
    the rerank to the pool's best rerank_factor x k, warps_per_query=4
    walks each query with four warps (beam search: lower latency),
    lists_per_step=1..4 walks it with one warp expanding that many lists per
    step (beam search, tensor-core distances: throughput), and
    filter_scan_mode picks the exact scan as in Index.search_batch_ex."""

    def __init__(self, index: Index, max_inflight: int = 4, max_batch_queries: int = 4096, memory_budget: int = 0,
                 precision: int = 0, filter_scan: float = 0.0, rerank_factor: int = 0, warps_per_query: int = 1,
                 lists_per_step: int = 0, filter_scan_mode: str = "auto"):
        self._h = None
        self._index = index  # keep the index alive
        cfg = _ServerConfig(max_inflight, max_batch_queries, memory_budget, precision,
                            int(round(filter_scan * 1000)), _rerank_factor(rerank_factor),
                            _warps_per_query(warps_per_query), _lists_per_step(lists_per_step),
                            _scan_mode(filter_scan_mode))
        h = C.c_void_p()
        _check(lib().hg_server_create(index._h, C.byref(cfg), C.byref(h)))
        self._h = h
        self._live = {}
        self.dim = index.dim

    def close(self):
        if getattr(self, "_h", None):
            lib().hg_server_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def _request(self, queries, k, ef, filter, keep):
        q = np.ascontiguousarray(queries, dtype=np.float32).reshape(-1, self.dim)
        out = np.empty(q.shape[0] * k, dtype=NEIGHBOR)
        fh = _FilterHolder(filter)
        keep.extend([q, out, fh])
        r = _Request(q.ctypes.data, q.shape[0], k, ef, 0, C.pointer(fh.struct) if fh.struct is not None else None,
                     out.ctypes.data)
        return r, out

    def submit(self, queries, k: int, ef: int = 0, filter=None) -> int:
        keep = []
        r, out = self._request(queries, k, ef, filter, keep)
        t = C.c_uint64()
        _check(lib().hg_server_submit(self._h, C.byref(r), C.byref(t)))
        self._live[t.value] = (keep, out, k)
        return t.value

    def wait(self, ticket: int):
        lat = C.c_double()
        try:
            _check(lib().hg_server_wait(self._h, ticket, C.byref(lat)))
        finally:
            keep, out, k = self._live.pop(ticket, (None, None, 1))
        return out.reshape(-1, k), lat.value

    def replay(self, requests, arrivals_s, latencies=False):
        """requests: list of (queries, k, ef, filter); arrivals_s: seconds from the
        call.  Returns (stats dict, list of result record arrays) and, with
        latencies=True, each request's latency in ms as a third item."""
        keep, outs = [], []
        arr = (_Request * len(requests))()
        for i, (q, k, ef, f) in enumerate(requests):
            r, out = self._request(q, k, ef, f, keep)
            arr[i] = r
            outs.append((out, k))
        at = np.ascontiguousarray(arrivals_s, dtype=np.float64)
        st = _ServerStats()
        lat = np.zeros(len(requests), dtype=np.float64)
        _check(lib().hg_server_replay_latencies(self._h, arr, at.ctypes.data, len(requests), C.byref(st),
                                                lat.ctypes.data))
        stats = {f: getattr(st, f) for f, _ in _ServerStats._fields_}
        res = [o.reshape(-1, k) for o, k in outs]
        return (stats, res, lat) if latencies else (stats, res)

