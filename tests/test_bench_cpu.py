"""bench.py's host-side arithmetic, checked without a GPU: the parity counts
(ids and distance bits), the operating-point choice (the smallest ef whose
recall reaches the target) and the algorithmic bytes behind the roofline
figure (the per-query traffic formula of the walk)."""
from __future__ import annotations

import subprocess
import sys
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(REPO))

import bench  # noqa: E402

REC = np.dtype([("label", "<u8"), ("distance", "<f4"), ("reserved", "<u4")])


def test_parity_counts_ids_and_distance_bits():
    a = np.zeros((3, 2), dtype=REC)
    a["label"] = [[1, 2], [3, 4], [5, 6]]
    a["distance"] = [[0.5, 1.0], [0.0, 2.0], [3.0, 4.0]]
    b = a.copy()
    assert bench.parity(a, b) == {"id_mismatches": 0, "distance_bit_mismatches": 0}
    b["label"][2, 1] = 7
    b["distance"][1, 0] = -0.0  # equal as floats, different bits
    b["distance"][0, 1] = np.nextafter(np.float32(1.0), np.float32(2.0))
    assert bench.parity(a, b) == {"id_mismatches": 1, "distance_bit_mismatches": 2}


def test_operating_point_is_the_smallest_ef_reaching_the_target():
    rows = [{"ef": 16, "recall_at_10": 0.90}, {"ef": 24, "recall_at_10": 0.951}, {"ef": 32, "recall_at_10": 0.97}]
    assert bench.first_at_target(rows)["ef"] == 24
    short = [{"ef": 16, "recall_at_10": 0.70}, {"ef": 24, "recall_at_10": 0.93}, {"ef": 32, "recall_at_10": 0.92}]
    assert bench.first_at_target(short)["ef"] == 24  # target never reached: the best row


def test_algorithmic_bytes_per_query():
    # counters per query: upper lists, upper distances, layer-0 lists,
    # layer-0 distances, visited, steps, rerank pool, tiers
    cnt = np.array([[3, 40, 50, 800, 0, 0, 40, 0], [1, 10, 20, 300, 0, 0, 40, 0]], dtype=np.uint64)
    dim, pd, k, M = 128, 128, 10, bench.M
    up, l0 = 4 * (1 + M), 4 * (1 + 2 * M)

    def per(c, row, rerank):
        return 4 * dim + c[0] * up + c[1] * row + c[2] * l0 + c[3] * row + k * 16 + (c[6] * 4 * pd if rerank else 0)

    fp32 = bench.algorithmic_bytes(cnt, dim, pd, k, {"precision": 0})
    assert fp32 == sum(per(c, 4 * pd, False) for c in cnt.astype(np.int64))
    beam16 = bench.algorithmic_bytes(cnt, dim, pd, k, {"precision": 1, "lists_per_step": 2})
    assert beam16 == sum(per(c, 2 * 128 + 8, True) for c in cnt.astype(np.int64))
    walk8 = bench.algorithmic_bytes(cnt, dim, pd, k, {"precision": 2})
    assert walk8 == sum(per(c, 128 + 4, True) for c in cnt.astype(np.int64))


def test_cli_parses_without_a_gpu():
    r = subprocess.run([sys.executable, str(REPO / "bench.py"), "--help"], capture_output=True, text=True,
                       timeout=120)
    assert r.returncode == 0
    for flag in ("--gpus", "--steps", "--warmup", "--impl", "--no-build"):
        assert flag in r.stdout
