"""Shared fixtures: the built library, the oracle, the golden fixtures and the
graphs rebuilt from the golden inputs with the library's single-threaded
builder (checked byte-for-byte against the reference's files)."""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parents[1]
GOLD = REPO / "tests" / "golden"
sys.path.insert(0, str(REPO / "hnsw-engine_gb300"))
sys.path.insert(0, str(REPO / "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu on a GB300)")


def sha256(path) -> str:
    return hashlib.sha256(Path(path).read_bytes()).hexdigest()


@pytest.fixture(scope="session")
def hg():
    """The hnswgpu module with libhnswgpu.so built (incrementally) in-tree.

    The golden fixtures were recorded by the reference on an x86-64 host in
    its AVX-512 order, so indexes start in that order on every host (an Arm
    host would otherwise default to NEON); tests of the NEON order set it
    themselves."""
    import build as gpubuild  # hnsw-engine_gb300/build.py

    gpubuild.build()
    import hnswgpu

    hnswgpu.set_distance_order("avx512")
    return hnswgpu


@pytest.fixture(scope="session")
def oracle():
    import pyoracle

    pyoracle.build()
    return pyoracle


@pytest.fixture(scope="session")
def golden():
    meta = json.loads((GOLD / "golden.json").read_text())
    arrays = dict(np.load(GOLD / "golden.npz"))
    return meta, arrays


def _case_data(name: str):
    import workloads

    if name == "c1":
        return workloads.int_mixture(20000, 128, 64, 1000), "l2", 16, 200
    if name == "c3s":
        return workloads.unit_mixture(4000, 100, 100, 200), "cosine", 16, 200
    if name == "c4s":
        return workloads.scaled_abs_normal(2000, 960, 100), "l2", 16, 200
    if name == "ip":
        d = np.load(GOLD / "ip_data.npz")
        return (d["base"], d["queries"]), "ip", 12, 100
    raise KeyError(name)


class GoldenGraphs:
    """Graph files of the golden cases, built once per session by the library."""

    def __init__(self, hg, golden, tmp: Path):
        self.hg, self.meta, self.tmp = hg, golden[0], tmp
        self._paths = {}
        self._data = {}

    def data(self, name):
        if name not in self._data:
            (base, q), metric, M, efc = _case_data(name)
            case = self.meta["cases"][name]
            assert hashlib.sha256(base.tobytes()).hexdigest() == case["base_sha"], f"{name}: base data drifted"
            assert hashlib.sha256(q.tobytes()).hexdigest() == case["query_sha"], f"{name}: query data drifted"
            self._data[name] = (base, q, metric, M, efc)
        return self._data[name]

    def path(self, name, deleted=False):
        key = (name, deleted)
        if key not in self._paths:
            base, _, metric, M, efc = self.data(name)
            ix = self.hg.Index(base.shape[1], metric, M, efc)
            ix.add(base, num_threads=1)
            p = self.tmp / f"{name}.idx"
            ix.save(p)
            self._paths[(name, False)] = p
            if name == "c3s":
                import workloads

                for lab in workloads.random_deletes(base.shape[0], 0.01, seed=2):
                    ix.mark_deleted(int(lab))
                pd = self.tmp / f"{name}_del.idx"
                ix.save(pd)
                self._paths[(name, True)] = pd
        return self._paths[key]


@pytest.fixture(scope="session")
def graphs(hg, golden, tmp_path_factory):
    return GoldenGraphs(hg, golden, tmp_path_factory.mktemp("graphs"))


def pytest_collection_modifyitems(config, items):
    # keep CPU-only runs free of CUDA initialisation: nothing to change, the
    # gpu marker is selected with -m.
    return
