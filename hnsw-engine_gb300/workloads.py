"""Seeded synthetic workloads with the shapes of the benchmark configurations.

The ann-benchmarks sets (SIFT-1M, GloVe-100, GIST) are not available offline;
these generators stand in for them with the same n, d, metric and value
distributions.  Every generator is a pure function of its seeds
(numpy ``default_rng``), so the same arrays come out on every machine.

Recipes (base vectors from seed 0, queries from seed 1, centres always from
the seed-0 stream so queries share the base's mixture):

* ``int_mixture``  -- Gaussian mixture, centres U[0,128)^d, sigma 20, rounded
  and clipped to [0,255], stored as float32.  Integer-valued float32 makes
  every squared-L2 partial sum exact (d <= 128), so distances do not depend on
  summation order.
* ``unit_mixture`` -- random unit centres plus N(0, 0.3^2) per dimension,
  renormalised (cosine workloads).
* ``scaled_abs_normal`` -- |N(0,1)| scaled per dimension by U[0.05, 1].
"""
from __future__ import annotations

import numpy as np


def int_mixture(n: int, d: int, clusters: int, nq: int, sigma: float = 20.0, qseed: int = 1):
    """Base (n, d) and query (nq, d) float32 arrays holding integers 0..255
    (queries from seed `qseed`, 1 for every benchmark workload)."""
    r0 = np.random.default_rng(0)
    centers = r0.uniform(0.0, 128.0, size=(clusters, d))
    c = r0.integers(0, clusters, size=n)
    base = np.clip(np.rint(centers[c] + r0.normal(0.0, sigma, size=(n, d))), 0, 255).astype(np.float32)
    r1 = np.random.default_rng(qseed)
    cq = r1.integers(0, clusters, size=nq)
    queries = np.clip(np.rint(centers[cq] + r1.normal(0.0, sigma, size=(nq, d))), 0, 255).astype(np.float32)
    return base, queries


def unit_mixture(n: int, d: int, clusters: int, nq: int, noise: float = 0.3, qseed: int = 1):
    """Unit-normalised mixture around random unit centres (cosine); queries
    from seed `qseed` (1 for every benchmark workload)."""
    r0 = np.random.default_rng(0)
    centers = r0.normal(size=(clusters, d))
    centers /= np.linalg.norm(centers, axis=1, keepdims=True)
    c = r0.integers(0, clusters, size=n)
    base = centers[c] + r0.normal(0.0, noise, size=(n, d))
    base /= np.linalg.norm(base, axis=1, keepdims=True)
    r1 = np.random.default_rng(qseed)
    cq = r1.integers(0, clusters, size=nq)
    queries = centers[cq] + r1.normal(0.0, noise, size=(nq, d))
    queries /= np.linalg.norm(queries, axis=1, keepdims=True)
    return base.astype(np.float32), queries.astype(np.float32)


def scaled_abs_normal(n: int, d: int, nq: int):
    """|N(0,1)| times a per-dimension scale drawn from U[0.05, 1]."""
    r0 = np.random.default_rng(0)
    scale = r0.uniform(0.05, 1.0, size=d)
    base = np.abs(r0.normal(size=(n, d))) * scale
    r1 = np.random.default_rng(1)
    queries = np.abs(r1.normal(size=(nq, d))) * scale
    return base.astype(np.float32), queries.astype(np.float32)


def label_filter_bits(num_labels: int, keep) -> np.ndarray:
    """BitsetFilter words (uint64, bit l of word l>>6) for labels where keep(l)."""
    labels = np.arange(num_labels, dtype=np.uint64)
    mask = np.asarray(keep(labels), dtype=bool)
    return mask_to_words(mask)


def mask_to_words(mask: np.ndarray) -> np.ndarray:
    """Pack a boolean mask over labels into little-endian uint64 words."""
    nbits = mask.shape[0]
    nwords = (nbits + 63) // 64
    padded = np.zeros(nwords * 64, dtype=bool)
    padded[:nbits] = mask
    by = np.packbits(padded.reshape(-1, 8), axis=1, bitorder="little").reshape(-1)
    return by.view(np.uint64).copy() if nwords else np.zeros(0, dtype=np.uint64)


def random_deletes(n: int, fraction: float, seed: int = 2) -> np.ndarray:
    """Labels to soft-delete: a uniform random `fraction` of arange(n)."""
    r = np.random.default_rng(seed)
    m = int(round(n * fraction))
    return np.sort(r.choice(n, size=m, replace=False)).astype(np.uint64)


def exact_knn_f64(base: np.ndarray, queries: np.ndarray, k: int, metric: str = "l2", block: int = 1024):
    """FP64 exact kNN (ids, distances) -- ties broken by label, as the reference does."""
    b = base.astype(np.float64)
    ids = np.empty((queries.shape[0], k), dtype=np.int64)
    dd = np.empty((queries.shape[0], k), dtype=np.float64)
    if metric == "cosine":
        b = b / np.maximum(np.linalg.norm(b, axis=1, keepdims=True), 1e-300)
    bn = (b * b).sum(1)
    for s in range(0, queries.shape[0], block):
        q = queries[s:s + block].astype(np.float64)
        if metric == "cosine":
            q = q / np.maximum(np.linalg.norm(q, axis=1, keepdims=True), 1e-300)
        if metric == "l2":
            d = (q * q).sum(1)[:, None] - 2.0 * (q @ b.T) + bn[None, :]
        else:
            d = 1.0 - q @ b.T
        part = np.argpartition(d, min(k, d.shape[1] - 1), axis=1)[:, :k + 1] if d.shape[1] > k else \
            np.tile(np.arange(d.shape[1]), (d.shape[0], 1))
        for i in range(d.shape[0]):
            cand = part[i]
            order = np.lexsort((cand, d[i, cand]))[:k]
            ids[s + i, :len(order)] = cand[order]
            dd[s + i, :len(order)] = d[i, cand[order]]
    return ids, dd


def recall_at_k(got: np.ndarray, truth: np.ndarray) -> float:
    """Mean |got_i ∩ truth_i| / k over queries (labels; -1/invalid never match;
    a row's labels are distinct)."""
    k = truth.shape[1]
    g = np.asarray(got, dtype=np.int64)[:, :k]
    t = np.asarray(truth, dtype=np.int64)
    hits = 0
    for s in range(0, g.shape[0], 8192):
        gg, tt = g[s:s + 8192], t[s:s + 8192]
        hits += int(((gg[:, :, None] == tt[:, None, :]) & (gg[:, :, None] >= 0)).any(2).sum())
    return hits / float(truth.shape[0] * k)
