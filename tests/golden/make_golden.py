"""Generate the golden fixtures from the reference hnsw-engine itself.

Run where the reference sources exist (they are compiled by
``make -C oracle ref`` into oracle/_ref/ref_driver):

    python tests/golden/make_golden.py

Every fixture is an output of the reference's own code: graphs built with its
single-threaded ``add_batch`` and written by its ``save`` (committed as small
files, or as a SHA-256 when large), ``search_batch`` / ``search`` results,
brute-force results, raw distance-kernel values per ISA, and the list of
corrupted files its ``load`` rejects.  The inputs are the seeded generators of
hnsw-engine_gb300/workloads.py, so tests regenerate them and check their
digests before comparing.
"""
from __future__ import annotations

import hashlib
import json
import os
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parents[2]
GOLD = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO / "hnsw-engine_gb300"))
import workloads  # noqa: E402

DRIVER = REPO / "oracle" / "_ref" / "ref_driver"
REC = np.dtype([("label", "<u8"), ("dist", "<f4")])


def sha(b: bytes) -> str:
    return hashlib.sha256(b).hexdigest()


def run(*args, env=None):
    subprocess.run([str(DRIVER), *map(str, args)], check=True, env=env)


def build(tmp: Path, name: str, base: np.ndarray, metric: str, M=16, efc=200, seed=100, labels=None) -> Path:
    vp = tmp / f"{name}.f32"
    base.astype(np.float32).tofile(vp)
    out = tmp / f"{name}.idx"
    extra = []
    if labels is not None:
        lp = tmp / f"{name}.lab"
        np.asarray(labels, dtype=np.uint64).tofile(lp)
        extra = [lp]
    run("build", vp, base.shape[0], base.shape[1], metric, M, efc, seed, 1, out, *extra)
    return out


def search(tmp: Path, idx: Path, queries: np.ndarray, k: int, ef: int, filt=None):
    qp = tmp / "q.f32"
    queries.astype(np.float32).tofile(qp)
    out = tmp / "res.bin"
    extra = []
    if filt is not None:
        fp = tmp / "filt.u64"
        filt[0].astype(np.uint64).tofile(fp)
        extra = [fp, filt[1]]
    run("search", idx, qp, queries.shape[0], k, ef, 8, out, *extra)
    r = np.fromfile(out, dtype=REC)
    return r["label"].reshape(queries.shape[0], k), r["dist"].reshape(queries.shape[0], k)


def search1(tmp: Path, idx: Path, q: np.ndarray, k: int, ef: int, filt=None):
    qp = tmp / "q1.f32"
    q.astype(np.float32).tofile(qp)
    out = tmp / "res1.bin"
    extra = []
    if filt is not None:
        fp = tmp / "filt1.u64"
        filt[0].astype(np.uint64).tofile(fp)
        extra = [fp, filt[1]]
    run("search1", idx, qp, k, ef, out, *extra)
    r = np.fromfile(out, dtype=REC)
    return r["label"], r["dist"]


def bf(tmp: Path, base, queries, k, metric, filt=None):
    bp, qp, out = tmp / "bfb.f32", tmp / "bfq.f32", tmp / "bf.bin"
    base.astype(np.float32).tofile(bp)
    queries.astype(np.float32).tofile(qp)
    extra = []
    if filt is not None:
        fp = tmp / "bff.u64"
        filt[0].astype(np.uint64).tofile(fp)
        extra = [fp, filt[1]]
    run("bf", bp, base.shape[0], base.shape[1], metric, qp, queries.shape[0], k, 8, out, *extra)
    r = np.fromfile(out, dtype=REC)
    return r["label"].reshape(queries.shape[0], k), r["dist"].reshape(queries.shape[0], k)


def delete(tmp: Path, idx: Path, labels: np.ndarray, out: Path, set_ef=None):
    lp = tmp / "del.u64"
    np.asarray(labels, dtype=np.uint64).tofile(lp)
    extra = [] if set_ef is None else [set_ef]
    run("delete", idx, lp, len(labels), out, *extra)


def ref_loads(path: Path, mmap: bool) -> bool:
    r = subprocess.run([str(DRIVER), "load", str(path), "1" if mmap else "0"], capture_output=True, text=True)
    return r.returncode == 0


def main():
    if not DRIVER.exists():
        subprocess.run(["make", "-s", "-C", str(REPO / "oracle"), "ref"], check=True)
    isa = subprocess.run([str(DRIVER), "isa"], capture_output=True, text=True, check=True).stdout.strip()
    meta = {"reference_isa": isa, "cases": {}}
    arrays = {}
    with tempfile.TemporaryDirectory() as td:
        tmp = Path(td)

        # ---- config 1: plain L2, n=20k d=128, 64-cluster integer mixture -----
        base, q = workloads.int_mixture(20000, 128, 64, 1000)
        idx = build(tmp, "c1", base, "l2")
        meta["cases"]["c1"] = {"n": 20000, "d": 128, "clusters": 64, "nq": 1000, "metric": "l2", "M": 16, "efc": 200,
                               "base_sha": sha(base.tobytes()), "query_sha": sha(q.tobytes()),
                               "index_sha": sha(idx.read_bytes()), "k": 10, "efs": [10, 20, 40, 80, 160]}
        for ef in [10, 20, 40, 80, 160]:
            lab, dist = search(tmp, idx, q, 10, ef)
            arrays[f"c1_ef{ef}_labels"] = lab.astype(np.int64)
            arrays[f"c1_ef{ef}_dists"] = dist
        # brute force ground truth on the same data (exact: integer data)
        lab, dist = bf(tmp, base, q[:200], 10, "l2")
        arrays["c1_bf_labels"] = lab.astype(np.int64)
        arrays["c1_bf_dists"] = dist

        # ---- config-3 shape, small: cosine d=100, filter label%10==0, 1% deleted
        n3, nq3 = 4000, 200
        base3, q3 = workloads.unit_mixture(n3, 100, 100, nq3)
        idx3 = build(tmp, "c3s", base3, "cosine")
        dels = workloads.random_deletes(n3, 0.01, seed=2)
        idx3d = tmp / "c3s_del.idx"
        delete(tmp, idx3, dels, idx3d)
        fw = workloads.label_filter_bits(n3, lambda l: l % 10 == 0)
        meta["cases"]["c3s"] = {"n": n3, "d": 100, "clusters": 100, "nq": nq3, "metric": "cosine", "M": 16,
                                "efc": 200, "base_sha": sha(base3.tobytes()), "query_sha": sha(q3.tobytes()),
                                "index_sha": sha(idx3.read_bytes()), "deleted_index_sha": sha(idx3d.read_bytes()),
                                "deleted_frac": 0.01, "groups": []}
        for k in (10, 100):
            for ef in (40, 160, 400):
                if ef < k:
                    continue
                for filtered in (False, True):
                    lab, dist = search(tmp, idx3d, q3, k, ef, (fw, n3) if filtered else None)
                    key = f"c3s_k{k}_ef{ef}_{'f' if filtered else 'u'}"
                    arrays[key + "_labels"] = lab.astype(np.int64)
                    arrays[key + "_dists"] = dist
                    meta["cases"]["c3s"]["groups"].append([k, ef, filtered])
        lab, dist = search(tmp, idx3, q3, 10, 40)  # no deletes: unfiltered variant
        arrays["c3s_nodel_k10_ef40_labels"] = lab.astype(np.int64)
        arrays["c3s_nodel_k10_ef40_dists"] = dist
        lab, dist = bf(tmp, base3, q3[:100], 10, "cosine", (fw, n3))
        arrays["c3s_bf_f_labels"] = lab.astype(np.int64)
        arrays["c3s_bf_f_dists"] = dist

        # ---- config-4 shape, small: float L2 d=960 ---------------------------
        base4, q4 = workloads.scaled_abs_normal(2000, 960, 100)
        idx4 = build(tmp, "c4s", base4, "l2")
        meta["cases"]["c4s"] = {"n": 2000, "d": 960, "nq": 100, "metric": "l2", "M": 16, "efc": 200,
                                "base_sha": sha(base4.tobytes()), "query_sha": sha(q4.tobytes()),
                                "index_sha": sha(idx4.read_bytes()), "efs": [40, 128]}
        for ef in (40, 128):
            lab, dist = search(tmp, idx4, q4, 10, ef)
            arrays[f"c4s_ef{ef}_labels"] = lab.astype(np.int64)
            arrays[f"c4s_ef{ef}_dists"] = dist
        lab, dist = bf(tmp, base4, q4[:50], 10, "l2")
        arrays["c4s_bf_labels"] = lab.astype(np.int64)
        arrays["c4s_bf_dists"] = dist

        # ---- inner product, d=33 (padded dim 48), M=12 -----------------------
        r = np.random.default_rng(5)
        centers = r.normal(0, 4, size=(16, 33))
        baseip = (centers[r.integers(0, 16, 3000)] + r.normal(size=(3000, 33))).astype(np.float32)
        qip = (centers[r.integers(0, 16, 100)] + r.normal(size=(100, 33))).astype(np.float32)
        idxip = build(tmp, "ip", baseip, "ip", M=12, efc=100)
        meta["cases"]["ip"] = {"n": 3000, "d": 33, "nq": 100, "metric": "ip", "M": 12, "efc": 100,
                               "base_sha": sha(baseip.tobytes()), "query_sha": sha(qip.tobytes()),
                               "index_sha": sha(idxip.read_bytes())}
        lab, dist = search(tmp, idxip, qip, 10, 100)
        arrays["ip_labels"] = lab.astype(np.int64)
        arrays["ip_dists"] = dist
        np.savez_compressed(GOLD / "ip_data.npz", base=baseip, queries=qip)

        # ---- small committed index files (edge cases and loader tests) --------
        small = {}
        # dim = 1, values 0..199 (test_index.cpp DimOne)
        b1 = np.arange(200, dtype=np.float32).reshape(200, 1)
        small["dim1"] = build(tmp, "dim1", b1, "l2")
        # identical vectors (IdenticalVectors)
        small["identical"] = build(tmp, "identical", np.full((300, 12), 0.5, dtype=np.float32), "l2")
        # empty index, dim 8
        small["empty"] = build(tmp, "empty", np.zeros((0, 8), dtype=np.float32), "l2")
        # five vectors, dim 4 (KLargerThanSizeAndEfClamp)
        r = np.random.default_rng(11)
        b5 = r.uniform(-1, 1, size=(5, 4)).astype(np.float32)
        small["five"] = build(tmp, "five", b5, "l2")
        # all deleted (AllDeleted)
        b20 = r.uniform(-1, 1, size=(20, 4)).astype(np.float32)
        alld = build(tmp, "all20", b20, "l2")
        small["alldeleted"] = tmp / "alldeleted.idx"
        delete(tmp, alld, np.arange(20), small["alldeleted"])
        # collinear points, every node reachable (ParallelBuildKeepsEveryNodeReachable)
        bcol = np.full((100, 128), 0.5, dtype=np.float32)
        bcol[:, 0] = np.arange(100)
        small["collinear"] = build(tmp, "collinear", bcol, "l2", seed=3)
        # non-identity labels, cosine, M=6 efc=40, one tombstone, ef default 33
        bl = r.normal(size=(300, 6)).astype(np.float32)
        labs = (1000 + 3 * np.arange(300)).astype(np.uint64)
        lidx = build(tmp, "labels", bl, "cosine", M=6, efc=40, labels=labs)
        small["labels"] = tmp / "labels_del.idx"
        delete(tmp, lidx, np.array([1003], dtype=np.uint64), small["labels"], set_ef=33)
        # mixed-data, M=8, dim 37, clustered, with two tombstones (persist round trip)
        bp = (np.random.default_rng(12).normal(0, 4, size=(8, 37))[r.integers(0, 8, 800)]
              + r.normal(size=(800, 37))).astype(np.float32)
        pidx = build(tmp, "persist", bp, "l2", M=8, efc=60)
        small["persist"] = tmp / "persist_del.idx"
        delete(tmp, pidx, np.array([5, 600], dtype=np.uint64), small["persist"])
        np.savez_compressed(GOLD / "small_data.npz", five=b5, all20=b20, labels=bl, labels_ids=labs, persist=bp)

        meta["small"] = {}
        for name, p in small.items():
            dst = GOLD / f"{name}.idx"
            dst.write_bytes(p.read_bytes())
            meta["small"][name] = sha(dst.read_bytes())

        # expected results on the small files
        lab, dist = search1(tmp, small["dim1"], np.array([42.2], dtype=np.float32), 3, 50)
        arrays["dim1_labels"], arrays["dim1_dists"] = lab.astype(np.int64), dist
        lab, dist = search1(tmp, small["identical"], np.full(12, 0.5, dtype=np.float32), 10, 64)
        arrays["identical_labels"], arrays["identical_dists"] = lab.astype(np.int64), dist
        lab, dist = search(tmp, small["empty"], np.zeros((1, 8), dtype=np.float32), 3, 10)
        arrays["empty_labels"], arrays["empty_dists"] = lab.astype(np.int64), dist
        lab, dist = search1(tmp, small["five"], b5[0], 50, 1)
        arrays["five_labels"], arrays["five_dists"] = lab.astype(np.int64), dist
        lab, dist = search1(tmp, small["alldeleted"], b20[0], 5, 10)
        arrays["alldeleted_labels"], arrays["alldeleted_dists"] = lab.astype(np.int64), dist
        lab, dist = search1(tmp, small["collinear"], bcol[0], 100, 200)
        arrays["collinear_all_labels"], arrays["collinear_all_dists"] = lab.astype(np.int64), dist
        allow = workloads.mask_to_words(np.isin(np.arange(100), [7, 99]))
        lab, dist = search1(tmp, small["collinear"], bcol[0], 10, 64, (allow, 100))
        arrays["collinear_f_labels"], arrays["collinear_f_dists"] = lab.astype(np.int64), dist
        ql = r.normal(size=(40, 6)).astype(np.float32)
        np.save(GOLD / "labels_queries.npy", ql)
        fl = workloads.mask_to_words(np.arange(2000) % 2 == 0)
        lab, dist = search(tmp, small["labels"], ql, 5, 0)  # ef 0 -> the saved default (33)
        arrays["labels_u_labels"], arrays["labels_u_dists"] = lab.astype(np.int64), dist
        lab, dist = search(tmp, small["labels"], ql, 5, 20, (fl, 2000))
        arrays["labels_f_labels"], arrays["labels_f_dists"] = lab.astype(np.int64), dist

        # ---- raw distance kernels, per ISA (pins the ISA emulations) ----------
        dims = [1, 7, 8, 9, 15, 16, 17, 31, 33, 63, 64, 65, 100, 112, 128, 960]
        rk = np.random.default_rng(21)
        meta["kernels"] = {"dims": dims, "count": 8, "isas": ["scalar", "avx2", "avx512"]}
        kin = {}
        for d in dims:
            kin[f"a{d}"] = rk.uniform(-2, 2, size=(8, d)).astype(np.float32)
            kin[f"b{d}"] = rk.uniform(-2, 2, size=(8, d)).astype(np.float32)
        np.savez_compressed(GOLD / "kernel_inputs.npz", **kin)
        for isa_name in ("scalar", "avx2", "avx512"):
            for d in dims:
                ap, bp_, op = tmp / "ka.f32", tmp / "kb.f32", tmp / "k.bin"
                kin[f"a{d}"].tofile(ap)
                kin[f"b{d}"].tofile(bp_)
                run("kernel", isa_name, ap, bp_, d, 8, op)
                arrays[f"kern_{isa_name}_{d}"] = np.fromfile(op, dtype=np.float32).reshape(8, 2)

        # ---- persistence fuzz: corruptions the reference's load rejects -------
        src = small["labels"].read_bytes()
        rf = np.random.default_rng(7)
        flips = [(i, int(rf.integers(0, 8))) for i in range(256)]
        flips += [(int(rf.integers(0, len(src))), int(rf.integers(0, 8))) for _ in range(300)]
        cuts = [0, 1, 7, 8, 100, 255, 256, 257, len(src) - 1] + [int(rf.integers(0, len(src))) for _ in range(40)]
        bad = tmp / "bad.idx"
        rejected_flips, rejected_cuts = [], []
        for pos, bit in flips:
            b = bytearray(src)
            b[pos] ^= 1 << bit
            bad.write_bytes(bytes(b))
            if not ref_loads(bad, False) and not ref_loads(bad, True):
                rejected_flips.append([pos, bit])
        for c in cuts:
            bad.write_bytes(src[:c])
            if not ref_loads(bad, False) and not ref_loads(bad, True):
                rejected_cuts.append(c)
        bad.write_bytes(src + b"\0")
        meta["fuzz"] = {"file": "labels.idx", "flips": rejected_flips, "cuts": rejected_cuts,
                        "appended_rejected": not ref_loads(bad, False),
                        "flips_tried": len(flips), "cuts_tried": len(cuts)}

    np.savez_compressed(GOLD / "golden.npz", **arrays)
    (GOLD / "golden.json").write_text(json.dumps(meta, indent=1, sort_keys=True) + "\n")
    print("wrote", GOLD / "golden.npz", os.path.getsize(GOLD / "golden.npz"), "bytes")


if __name__ == "__main__":
    main()
