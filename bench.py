"""Benchmark of the batched HNSW query path on GB300.

Headline (the metric's configuration): QPS at recall@10 >= 0.95 on 1M x 128
L2.  n = 1,000,000 vectors from a 1,024-cluster integer Gaussian mixture
(seed 0), M = 16, ef_construction = 200, the graph built by the reference's
own add_batch (its C++ library compiled on this host) and loaded by both
sides from the same file; 100,000 queries (seed 1) per step, k = 10.  Every
form runs at the smallest ef of a fixed list whose recall@10 on the first
10,000 queries reaches 0.95 (exact k-NN ground truth).  The data are seeded
synthetic stand-ins with SIFT-1M's shape (the ann-benchmarks sets are not
available offline).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  `value`: QPS of the fastest compressed form
(FP16 / FP8 traversal + exact FP32 rerank, batched) with queries already in
HBM, CUDA events on the launch stream; `e2e`: the same form through the host
C ABI with pinned host buffers, copies inside the timed region;
`config.plain_fp32`: the plain FP32 search_batch (the reference's algorithm,
id-exact) measured the same way.  `cpu_baseline` and `--impl reference` time
the reference's own Index::search_batch on the host cores.  Secondary blocks:
`batched_200k` (mixed ef in one launch; the tensor-core brute force),
`filtered_200k` (cosine with filters and deletes, mixed k / ef),
`serving` (continuous batching at 1M: p50 / p99 / p999), `precision`
(d = 960: FP32 / FP16 / FP8 error and recall), `build` (the graph linked on
the GPU against the reference's add_batch), `load` (file to searchable
device graph).  Every block compares the plain GPU answers with the
reference's on the same graph file (id and distance-bit mismatches).
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO / "hnsw-engine_gb300"))
sys.path.insert(0, str(REPO / "oracle"))

METRIC = "QPS at recall@10≥0.95 (served/batched vs plain GPU, same GB300); p50/p99 ms"
M, EFC = 16, 200
HEAD_N, HEAD_DIM, HEAD_CLUSTERS, HEAD_NQ, HEAD_K = 1_000_000, 128, 1024, 100_000, 10
HEAD_EFS = (16, 24, 32, 40, 48, 56, 64, 80, 96, 128, 160, 256)
RECALL_TARGET = 0.95
RECALL_SAMPLE = 10_000
REF_STEP_QUERIES = 20_000  # reference arm: queries per timed step (a bounded sample)
WORKLOAD = (f"l2-1M: n={HEAD_N} d={HEAD_DIM} (1,024-cluster integer mixture) M={M} efC={EFC}, graph from the "
            f"reference's add_batch; {HEAD_NQ} queries/step, k={HEAD_K}, each form at the smallest ef in "
            f"{list(HEAD_EFS)} with recall@10 >= {RECALL_TARGET} on the first {RECALL_SAMPLE} queries")
# GPU forms.  fp32_plain is the reference's algorithm (id-exact); the others
# walk compressed rows and rerank the best 4k of their pool in exact FP32.
FORMS = [
    ("fp32_plain", dict(precision=0)),
    ("fp16_beam2", dict(precision=1, rerank_factor=4, lists_per_step=2)),
    ("fp8_beam2", dict(precision=2, rerank_factor=4, lists_per_step=2)),
    ("fp16_beam4", dict(precision=1, rerank_factor=4, lists_per_step=4)),
    ("fp8_walk", dict(precision=2, rerank_factor=4)),
    ("fp8_4warps", dict(precision=2, rerank_factor=4, warps_per_query=4)),
]
# DRAM bytes (read + write) of one launch of the headline kernel (the FP16
# beam walk at ef 48) over the 100,000-query batch, from an ncu capture:
# 18.052 GB read + 0.143 GB written
HEAD_DRAM_BYTES = 18_195_270_000


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# ---------------------------------------------------------------------------
# graphs: the reference's add_batch, cached per host so both arms load one file
# ---------------------------------------------------------------------------
def cache_dir() -> Path:
    d = Path(os.environ.get("HNSW_BENCH_CACHE") or (Path(tempfile.gettempdir()) / "hnsw-gb300-bench"))
    d.mkdir(parents=True, exist_ok=True)
    return d


def bench_graph(tag: str, base: np.ndarray, metric: str = "l2"):
    """(path, seconds, 'built' | 'cached'): the reference's add_batch over base
    (all host threads), saved in its file format; reused when the same data
    were built before on this host."""
    import refcore

    h = hashlib.sha256()
    h.update(f"{tag}|{metric}|{M}|{EFC}|{base.shape}".encode())
    h.update(base[:: max(1, base.shape[0] // 4096)].tobytes())
    path = cache_dir() / f"{tag}-{h.hexdigest()[:16]}.idx"
    if path.exists():
        try:
            refcore.RefIndex(path)  # loads and validates (checksums)
            return path, 0.0, "cached"
        except Exception:  # noqa: BLE001 - rebuild a damaged file
            path.unlink()
    tmp = path.with_suffix(f".tmp{os.getpid()}")
    t0 = time.time()
    refcore.build(base, tmp, metric=metric, M=M, ef_construction=EFC, threads=0)
    os.replace(tmp, path)
    return path, time.time() - t0, "built"


def head_workload():
    import workloads

    return workloads.int_mixture(HEAD_N, HEAD_DIM, HEAD_CLUSTERS, HEAD_NQ)


def first_at_target(rows):
    """Smallest-ef row whose recall reaches the target (else the best row)."""
    for r in rows:
        if r["recall_at_10"] >= RECALL_TARGET:
            return r
    return max(rows, key=lambda r: r["recall_at_10"])


class Clocks:
    """nvidia-smi samples during the timed region (query only)."""

    def __init__(self, index: int = 0):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for line in Path(self.path).read_text().splitlines():
                f = [x.strip() for x in line.split(",")]
                if len(f) < 9:
                    continue
                try:
                    sm.append(float(f[1]))
                    mx = max(mx, float(f[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, f[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
        except OSError:
            pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = REPO / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def algorithmic_bytes(cnt: np.ndarray, dim: int, pd: int, k: int, kw: dict) -> float:
    """Bytes the walk must move per batch: the query, upper / layer-0 lists
    (68 / 132 B per list, the file's records), one row per distance (FP32
    4 pd; FP16 2 x 128 + 8 B row scale and norm on the beam walk; FP8 128 + 8 B
    on the beam walk, 128 + 4 B on the others), the exact rerank's FP32 rows
    and the output."""
    prec = kw.get("precision", 0)
    beam = kw.get("lists_per_step", 0) > 0
    row = {0: 4 * pd, 1: 2 * 128 + (8 if beam else 0), 2: 128 + (8 if beam else 4)}[prec]
    up_list, l0_list = 4 * (1 + M), 4 * (1 + 2 * M)
    per_q = 4 * dim + cnt[:, 0] * up_list + cnt[:, 1] * row + cnt[:, 2] * l0_list + cnt[:, 3] * row + k * 16
    if prec:
        per_q = per_q + cnt[:, 6] * 4 * pd
    return float(per_q.sum())


def launches_per_step(kw: dict) -> int:
    """Kernels one batch enqueues in these forms: the ef-bucketing kernel, one
    persistent walk (all queries, largest ef first) and the rerun pass."""
    return 3


# ---------------------------------------------------------------------------
# reference (CPU) helpers
# ---------------------------------------------------------------------------
def ref_time_batches(rx, batches, threads):
    """Wall seconds of one search_batch call per (queries, k, ef, filter) batch."""
    t0 = time.perf_counter()
    outs = [rx.search_batch(q, k, ef, threads=threads, filt=f) for q, k, ef, f in batches]
    return time.perf_counter() - t0, outs


def host_cpu():
    try:
        for line in Path("/proc/cpuinfo").read_text().splitlines():
            if line.lower().startswith(("model name", "cpu part")):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return os.uname().machine


def parity(gpu, ref):
    return {"id_mismatches": int((gpu["label"] != ref["label"]).sum()),
            "distance_bit_mismatches": int((gpu["distance"].view(np.uint32) != ref["distance"].view(np.uint32)).sum())}


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
def run_ours(args, rank, world, local):
    import torch

    import hnswgpu
    import refcore
    import workloads

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    base, queries = head_workload()
    gpath, build_s, build_how = bench_graph("l2-1m", base)
    ix = hnswgpu.Index.load(gpath)
    ix.set_device(local)
    pd = -(-HEAD_DIM // 16) * 16

    # ground truth of the recall sample: exact k-NN on the GPU (integer data:
    # FP32 is exact), pinned against the reference's brute force on a sample
    sample = queries[:RECALL_SAMPLE]
    bf = hnswgpu.BruteForceIndex(HEAD_DIM, "l2")
    bf.add(base)
    gt = bf.search_raw(sample, HEAD_K)["label"].astype(np.int64)
    del bf
    ref_bf = refcore.bruteforce(base, sample[:256], HEAD_K, threads=0)["label"].astype(np.int64)
    gt_pin = int((ref_bf != gt[:256]).sum())

    # operating point of every form: the smallest ef reaching the recall target
    sweep = {}
    for name, kw in FORMS:
        rows = []
        for ef in HEAD_EFS:
            got = ix.search_batch_ex(sample, HEAD_K, ef, **kw)["label"].astype(np.int64)
            rows.append({"ef": ef, "recall_at_10": round(workloads.recall_at_k(got, gt), 4)})
            if rows[-1]["recall_at_10"] >= RECALL_TARGET:
                break
        sweep[name] = rows

    stream = torch.cuda.Stream(device=dev)
    q_d = torch.from_numpy(queries).to(dev)
    out_d = torch.empty((HEAD_NQ, HEAD_K, 4), dtype=torch.int32, device=dev)  # 16-byte records
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # > L2 (129 MB)

    use_graph = args.launch == "graph"

    def step(kw, ef):
        ix.search_device(q_d.data_ptr(), HEAD_NQ, HEAD_K, ef, out_d.data_ptr(), stream.cuda_stream,
                         graph=use_graph, **kw)

    def timed(kw, ef, warmup, steps, clocks=None, nvtx=None):
        """Per-step device milliseconds (CUDA events on the launch stream);
        nvtx names a range around the timed steps (for a profiler's filter)."""
        with torch.cuda.stream(stream):
            for _ in range(warmup):
                flush.zero_()
                step(kw, ef)
            torch.cuda.synchronize()
            if world > 1:
                torch.distributed.barrier()
            torch.cuda.synchronize()
            ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
            if clocks:
                clocks.__enter__()
            if nvtx:
                torch.cuda.nvtx.range_push(nvtx)
            for i in range(steps):
                flush.zero_()
                ev[i][0].record(stream)
                step(kw, ef)
                ev[i][1].record(stream)
            torch.cuda.synchronize()
            if nvtx:
                torch.cuda.nvtx.range_pop()
            if clocks:
                clocks.__exit__()
        return [a.elapsed_time(b) for a, b in ev]

    # every form at its operating point (a short timing), then the headline
    table = {}
    for name, kw in FORMS:
        op = first_at_target(sweep[name])
        ms = timed(kw, op["ef"], 2, 3)
        table[name] = {"ef": op["ef"], "recall_at_10": op["recall_at_10"],
                       "qps": round(HEAD_NQ / (statistics.median(ms) / 1e3), 1), "sweep": sweep[name]}
    compressed = [n for n, _ in FORMS if n != "fp32_plain" and table[n]["recall_at_10"] >= RECALL_TARGET]
    head = max(compressed, key=lambda n: table[n]["qps"]) if compressed else "fp32_plain"
    head_kw = dict(FORMS)[head]
    head_ef = table[head]["ef"]
    plain_kw = dict(FORMS)["fp32_plain"]
    plain_ef = table["fp32_plain"]["ef"]

    clocks = Clocks(local)
    head_ms = timed(head_kw, head_ef, args.warmup, args.steps, clocks, nvtx="head_timed")
    plain_ms = timed(plain_kw, plain_ef, args.warmup, args.steps, nvtx="plain_timed")
    dev_ms = sum(head_ms)
    plain_dev_ms = sum(plain_ms)

    # e2e through the host C ABI: pinned queries in, pinned records out
    q_pin = torch.from_numpy(queries).pin_memory()
    out_pin = torch.empty((HEAD_NQ, HEAD_K, 4), dtype=torch.int32).pin_memory()
    qn = q_pin.numpy()
    on = out_pin.numpy().view(hnswgpu.NEIGHBOR).reshape(-1)
    e2e_ms = []
    with torch.cuda.stream(stream):
        for i in range(args.warmup + args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            ix.search_batch_ex(qn, HEAD_K, head_ef, stream=stream.cuda_stream, out=on, **head_kw)
            b.record(stream)
            torch.cuda.synchronize()
            if i >= args.warmup:
                e2e_ms.append(a.elapsed_time(b))
    e2e_total = sum(e2e_ms)
    # the device-resident batch answers as the host call does
    step(head_kw, head_ef)
    torch.cuda.synchronize()
    dev_rec = out_d.cpu().numpy().view(hnswgpu.NEIGHBOR).reshape(HEAD_NQ, HEAD_K)
    if not np.array_equal(dev_rec["label"], on.reshape(HEAD_NQ, HEAD_K)["label"]):
        raise RuntimeError("device-resident batch differs from the host-call batch")

    # traversal counters of the headline form (untimed) -> algorithmic bytes
    _, cnt = ix.search_batch_ex(queries, HEAD_K, head_ef, counters=True, **head_kw)
    alg_bytes = algorithmic_bytes(cnt, HEAD_DIM, pd, HEAD_K, head_kw)

    if world > 1:  # the job's time is the slowest replica's
        import replicas

        dev_ms, e2e_total = replicas.max_over_ranks(dev_ms), replicas.max_over_ranks(e2e_total)
        plain_dev_ms = replicas.max_over_ranks(plain_dev_ms)
    qps = world * HEAD_NQ * args.steps / (dev_ms / 1e3)
    e2e_qps = world * HEAD_NQ * args.steps / (e2e_total / 1e3)
    plain_qps = world * HEAD_NQ * args.steps / (plain_dev_ms / 1e3)
    per_launch_ms = dev_ms / args.steps
    peak, peak_kind = measured_peaks()
    achieved = alg_bytes / (per_launch_ms / 1e3) / 1e9
    prec = head_kw.get("precision", 0)
    result = {
        "metric": METRIC, "value": round(qps, 1), "unit": "queries/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(per_launch_ms, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": {0: "f32", 1: "f16", 2: "fp8-e4m3"}[prec],
        "data": "synthetic (seeded 1,024-cluster integer Gaussian mixture, SIFT-1M shape)",
        "config": {"workload": WORKLOAD, "global_batch": world * HEAD_NQ, "form": head, "form_options": head_kw,
                   "ef": head_ef, "recall_at_10": table[head]["recall_at_10"],
                   "plain_fp32": {"ef": plain_ef, "recall_at_10": table["fp32_plain"]["recall_at_10"],
                                  "qps": round(plain_qps, 1), "ms_per_step": round(plain_dev_ms / args.steps, 4)},
                   "compressed_over_plain": round(qps / plain_qps, 3),
                   "forms": table, "l2_flush": "256 MiB write before every timed step (the graph and rows "
                                                "also exceed the 129 MB L2)",
                   "launch": ("one CUDA-graph replay" if use_graph else "kernel launches") +
                             " per step: bucket kernel, one persistent walk, rerun pass",
                   "parallelism": f"replicas x{world} (queries per replica fixed)",
                   "graph": {"source": "reference add_batch (all host threads), FORMAT v1 file",
                             "seconds": round(build_s, 1), "how": build_how},
                   "ground_truth": {"kind": "GPU brute force, exact on integer data",
                                    "mismatches_vs_reference_bruteforce_256q": gt_pin},
                   "mean_l0_lists": round(float(cnt[:, 2].mean()), 2),
                   "mean_l0_distances": round(float(cnt[:, 3].mean()), 2)},
        "e2e": {"value": round(e2e_qps, 1), "unit": "queries/s",
                "h2d_bytes_per_step": int(HEAD_NQ * HEAD_DIM * 4), "d2h_bytes_per_step": int(HEAD_NQ * HEAD_K * 16)},
        "gpu_launches": launches_per_step(head_kw) * args.steps,
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": HEAD_DRAM_BYTES,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of the headline walk "
                                       "(one launch over the batch)",
                     "peak_source": peak_kind, "algorithmic_bytes_per_launch": int(alg_bytes),
                     "kernel": "beam_kernel" if head_kw.get("lists_per_step") else "search_kernel"},
        "clocks": clocks.summary(),
    }
    if rank == 0 and world == 1:
        result["cpu_baseline"] = cpu_baseline(ix, gpath, queries, plain_ef)
        if not args.no_build:
            result["build"] = run_build(ix, base, sample, gt, build_s, build_how)
        del ix
        if not args.no_batched:
            result["batched_200k"] = run_batched_200k(local, use_graph)
            result["filtered_200k"] = run_filtered_200k(local)
        if not args.no_serving:
            result["serving"] = run_serving(local, gpath)
        if not args.no_precision:
            result["precision"] = run_precision(local)
        result["load"] = run_load(gpath, queries[:1])
    return result


def run_build(ix_ref, base, sample, gt, ref_s, ref_how):
    """Graph construction on the GPU (Index.add_gpu) over the headline's 1M
    rows, against the reference's add_batch on all host threads (timed when
    the bench built the file in this run): wall time, and recall@10 of the
    plain FP32 walk on both graphs at several ef over the recall sample."""
    import hnswgpu
    import workloads

    def build(**kw):
        g = hnswgpu.Index(HEAD_DIM, "l2", M, EFC)
        t = time.perf_counter()
        st = g.add_gpu(base, **kw)
        return g, time.perf_counter() - t, st

    g, wall, st = build()
    gp, wall_p, st_p = build(wave_fraction=0.1, peers=True)
    rows = []
    for ef in (16, 32, 48, 96):
        r_ref = workloads.recall_at_k(ix_ref.search_raw(sample, HEAD_K, ef)["label"].astype(np.int64), gt)
        r_gpu = workloads.recall_at_k(g.search_raw(sample, HEAD_K, ef)["label"].astype(np.int64), gt)
        r_peer = workloads.recall_at_k(gp.search_raw(sample, HEAD_K, ef)["label"].astype(np.int64), gt)
        rows.append({"ef": ef, "recall_at_10_reference_graph": round(r_ref, 4),
                     "recall_at_10_gpu_graph": round(r_gpu, 4), "recall_at_10_gpu_graph_peers": round(r_peer, 4)})
    del g, gp
    return {"workload": f"the headline rows: n={HEAD_N} d={HEAD_DIM} M={M} efC={EFC}",
            "gpu_add_batch_s": round(wall, 3), "gpu_linking_s": round(st["seconds"], 3), "waves": st["waves"],
            "dropped_proposals": st["dropped_proposals"],
            "gpu_peers": {"options": "wave_fraction 0.1, peer linking", "add_batch_s": round(wall_p, 3),
                          "linking_s": round(st_p["seconds"], 3), "waves": st_p["waves"]},
            "reference_add_batch_s": round(ref_s, 2) if ref_how == "built" else None,
            "reference_threads": os.cpu_count(),
            "note": "add_batch_s covers the host store, the upload, the linking and the download; "
                    "recall of the plain walk, ground truth exact k-NN",
            "recall": rows}


def run_load(gpath, q1):
    """Load time of the headline graph file (FORMAT v1, page cache warm) until
    the graph can be searched on the GPU: Index.load then the upload on the
    first search, against Index.load(device=0), which streams the sections
    to the device while it reads and hashes them.  Median of 3, seconds."""
    import hnswgpu

    size = os.path.getsize(gpath)

    def once(mmap, device):
        t = time.perf_counter()
        ix = hnswgpu.Index.load(gpath, mmap, device=device)
        t_read = time.perf_counter() - t
        ix.search_raw(q1, 10, 48)  # the upload (if not done yet) and one query
        t_all = time.perf_counter() - t
        del ix
        return t_read, t_all

    out = {"file_bytes": size, "cache": "warm (the file was just read)"}
    for mmap in (False, True):
        for name, device in (("load_then_upload", None), ("streamed", 0)):
            runs = sorted((once(mmap, device) for _ in range(3)), key=lambda r: r[1])
            t_read, t_all = runs[1]
            out[f"{name}{'_mmap' if mmap else ''}"] = {"load_s": round(t_read, 3), "searchable_s": round(t_all, 3)}
    return out


def cpu_baseline(ix, gpath, queries, ef):
    """The reference's own search_batch on the host cores (all threads) at the
    plain path's operating ef, over the whole batch, and the plain GPU path's
    answers compared with it: ids and distance bits."""
    import refcore

    threads = os.cpu_count() or 1
    rx = refcore.RefIndex(gpath)
    rx.search_batch(queries[:2000], HEAD_K, ef, threads=threads)  # warm-up
    t0 = time.perf_counter()
    ref = rx.search_batch(queries, HEAD_K, ef, threads=threads)
    el = time.perf_counter() - t0
    gpu = ix.search_raw(queries, HEAD_K, ef)
    return {"value": round(HEAD_NQ / el, 1), "unit": "queries/s", "cores": threads, "kind": "reference",
            "sample": f"all {HEAD_NQ} queries of the batch in one reference search_batch call at ef={ef} "
                      f"(the plain form's operating point), {threads} threads, simd {refcore.isa()}, "
                      f"host {host_cpu()}",
            "parity_vs_plain_gpu": {"queries": HEAD_NQ, **parity(gpu, ref)}}


# ---------------------------------------------------------------------------
# batched L2 at 200k: per-query ef in one persistent launch
# ---------------------------------------------------------------------------
B2_N, B2_CLUSTERS, B2_NQ = 200_000, 256, 10_000
B2_EFS = (10, 20, 40, 80, 160, 320)


def run_batched_200k(local, use_graph=True):
    """200,000 x 128 (256 clusters), 10,000 queries with ef drawn per query from
    {10..320}, k = 10: one persistent launch on the GPU (plain FP32) against the
    reference's search_batch grouped per ef; ids and distances compared."""
    import torch

    import hnswgpu
    import refcore
    import workloads

    base, queries = workloads.int_mixture(B2_N, HEAD_DIM, B2_CLUSTERS, B2_NQ)
    efs = np.random.default_rng(3).choice(np.array(B2_EFS, dtype=np.uint32), size=B2_NQ)
    gpath, build_s, how = bench_graph("l2-200k", base)
    ix = hnswgpu.Index.load(gpath)
    ix.set_device(local)
    dev = torch.device("cuda", local)
    _, sample = workloads.int_mixture(B2_N, HEAD_DIM, B2_CLUSTERS, B2_NQ, qseed=2)
    sample_efs = np.random.default_rng(4).choice(np.array(B2_EFS, dtype=np.uint32), B2_NQ)
    ix.autotune(sample, k=HEAD_K, ef_max=int(efs.max()), precision=0, ef_per_query=sample_efs)
    stream = torch.cuda.Stream(device=dev)
    q_d = torch.from_numpy(queries).to(dev)
    ef_d = torch.from_numpy(efs.astype(np.int32)).to(dev)
    out_d = torch.empty((B2_NQ, HEAD_K, 4), dtype=torch.int32, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    ms = []
    with torch.cuda.stream(stream):
        for i in range(8):
            flush.zero_()
            if i == 3:
                torch.cuda.nvtx.range_push("b200_timed")
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            ix.search_device(q_d.data_ptr(), B2_NQ, HEAD_K, int(efs.max()), out_d.data_ptr(), stream.cuda_stream,
                             ef_ptr=ef_d.data_ptr(), graph=use_graph)
            b.record(stream)
            torch.cuda.synchronize()
            if i >= 3:
                ms.append(a.elapsed_time(b))
        torch.cuda.nvtx.range_pop()
    gpu = out_d.cpu().numpy().view(hnswgpu.NEIGHBOR).reshape(B2_NQ, HEAD_K)
    # the allocation-free entry point beside the allocating one (one ef, 80)
    noalloc = {}
    for name, call in (("search_batch", ix.search_device), ("noalloc", ix.search_noalloc)):
        t = []
        with torch.cuda.stream(stream):
            for i in range(5):
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                call(q_d.data_ptr(), B2_NQ, HEAD_K, 80, out_d.data_ptr(), stream.cuda_stream)
                b.record(stream)
                torch.cuda.synchronize()
                if i >= 2:
                    t.append(a.elapsed_time(b))
        noalloc[name + "_qps"] = round(B2_NQ / (statistics.median(t) / 1e3), 1)
    bf = hnswgpu.BruteForceIndex(HEAD_DIM, "l2")
    bf.add(base)
    gt = bf.search_raw(queries, HEAD_K)["label"].astype(np.int64)
    # the tensor-core brute force itself: host calls (copies, bound pass,
    # scan, select and exact rerank), median of 5
    bf_ms = []
    for _ in range(5):
        t = time.perf_counter()
        bf.search_raw(queries, HEAD_K)
        bf_ms.append((time.perf_counter() - t) * 1e3)
    bf_ms = statistics.median(bf_ms)
    bf_path = bf.last_path
    del bf
    threads = os.cpu_count() or 1
    rx = refcore.RefIndex(gpath)
    groups = [np.nonzero(efs == e)[0] for e in B2_EFS]
    batches = [(queries[g], HEAD_K, int(e), None) for g, e in zip(groups, B2_EFS)]
    ref_time_batches(rx, batches, threads)  # warm-up
    el, outs = ref_time_batches(rx, batches, threads)
    ref = np.empty((B2_NQ, HEAD_K), dtype=refcore.NEIGHBOR)
    for g, o in zip(groups, outs):
        ref[g] = o
    return {"workload": f"batched-L2-200k: n={B2_N} d={HEAD_DIM} M={M} efC={EFC} (reference add_batch), {B2_NQ} "
                        f"queries, per-query ef U{list(B2_EFS)}, k={HEAD_K}, one persistent launch (plain FP32)",
            "graph_seconds": round(build_s, 1), "graph": how,
            "qps": round(B2_NQ / (statistics.median(ms) / 1e3), 1), "ms_per_batch": round(statistics.median(ms), 4),
            "recall_at_10": round(workloads.recall_at_k(gpu["label"].astype(np.int64), gt), 4),
            "reference_qps": round(B2_NQ / el, 1),
            "noalloc": {**noalloc, "ef": 80, "note": "device-resident batch; the allocation-free call runs on a "
                                                      "fixed 48 warps"},
            "reference": f"search_batch per ef group, {threads} threads, simd {refcore.isa()}",
            "parity_vs_reference": {"queries": B2_NQ, **parity(gpu, ref)},
            "bruteforce": {"what": f"exact k-NN of the {B2_NQ} queries over the {B2_N} rows, k={HEAD_K}, one host "
                                   f"call (copies included), median of 5",
                           "ms": round(bf_ms, 3), "path": "tensor cores" if bf_path == 2 else "CUDA-core scan",
                           "tflops_effective": round(2.0 * B2_NQ * B2_N * HEAD_DIM / (bf_ms / 1e3) / 1e12, 1)}}


# ---------------------------------------------------------------------------
# cosine with filters and deletes at 200k: per-query k / ef / filter
# ---------------------------------------------------------------------------
C3_N, C3_DIM, C3_CENTERS, C3_NQ = 200_000, 100, 1000, 10_000
C3_EFS, C3_KS = (40, 100, 200, 400), (10, 100)


def run_filtered_200k(local):
    """200,000 x 100 unit vectors (cosine), 1% of the labels deleted (seed 2),
    10,000 queries, half filtered to label % 10 == 0, k in {10, 100} and ef in
    {40..400} per query: one GPU call (plain FP32) against the reference's
    search_batch, one call per (filtered, k, ef) group; ids and distances
    compared, recall@10 against exact k-NN over the allowed live rows."""
    import hnswgpu
    import refcore
    import workloads

    base, queries = workloads.unit_mixture(C3_N, C3_DIM, C3_CENTERS, C3_NQ)
    gpath, build_s, how = bench_graph("cos-200k", base, "cosine")
    dels = workloads.random_deletes(C3_N, 0.01, seed=2)
    keep = np.arange(C3_N) % 10 == 0
    fw = workloads.mask_to_words(keep)
    rng = np.random.default_rng(3)
    filt = rng.random(C3_NQ) < 0.5
    ks = rng.choice(np.array(C3_KS, dtype=np.uint32), C3_NQ)
    efs = rng.choice(np.array(C3_EFS, dtype=np.uint32), C3_NQ)
    fsel = np.where(filt, 0, -1).astype(np.int32)
    kmax = max(C3_KS)
    ix = hnswgpu.Index.load(gpath)
    ix.set_device(local)
    for lab in dels:
        ix.mark_deleted(int(lab))
    # launch shapes tuned on other queries of the same process (seed 2; the
    # tuner takes per-query ef, not filters)
    _, sample = workloads.unit_mixture(C3_N, C3_DIM, C3_CENTERS, 4096, qseed=2)
    t = time.perf_counter()
    ix.autotune(sample, k=max(C3_KS), ef_max=max(C3_EFS), precision=0,
                ef_per_query=np.random.default_rng(4).choice(np.array(C3_EFS, dtype=np.uint32), 4096))
    tune_s = time.perf_counter() - t
    bits = [hnswgpu.Bitset(fw, C3_N)]
    times = []
    for i in range(4):  # the first call uploads the graph and warms up
        t = time.perf_counter()
        rec = ix.search_batch_ex(queries, kmax, ef_per_query=efs, k_per_query=ks, filters=bits, filter_of_query=fsel)
        if i:
            times.append(time.perf_counter() - t)
    gpu_s = statistics.median(times)

    rx = refcore.RefIndex(gpath)
    for lab in dels:
        rx.mark_deleted(int(lab))
    rbits = refcore.Bitset(fw, C3_N)
    threads = os.cpu_count() or 1
    groups, batches = [], []
    for f in (False, True):
        for k in C3_KS:
            for ef in C3_EFS:
                g = np.nonzero((filt == f) & (ks == k) & (efs == ef))[0]
                if g.size:
                    groups.append((g, k))
                    batches.append((queries[g], int(k), int(ef), rbits if f else None))
    ref_time_batches(rx, batches, threads)  # warm-up
    el, outs = ref_time_batches(rx, batches, threads)
    ids = dist = 0
    for (g, k), o in zip(groups, outs):
        got = rec[g, :k]
        ids += int((got["label"] != o["label"]).sum())
        dist += int((got["distance"].view(np.uint32) != o["distance"].view(np.uint32)).sum())
    # recall@10 against exact k-NN over the rows each query may return
    alive = np.ones(C3_N, dtype=bool)
    alive[dels.astype(np.int64)] = False
    bf = hnswgpu.BruteForceIndex(C3_DIM, "cosine")
    bf.add(base)
    hit = 0
    for f in (False, True):
        g = np.nonzero(filt == f)[0]
        gt = bf.search_raw(queries[g], 10, filter=alive & keep if f else alive)["label"].astype(np.int64)
        hit += workloads.recall_at_k(rec[g, :10]["label"].astype(np.int64), gt) * g.size
    del bf
    return {"workload": f"cosine-200k: n={C3_N} d={C3_DIM} unit vectors ({C3_CENTERS} centres, noise 0.3) M={M} "
                        f"efC={EFC} (reference add_batch), 1% deleted, {C3_NQ} queries, half filtered to "
                        f"label % 10 == 0, k in {list(C3_KS)}, ef in {list(C3_EFS)} per query",
            "graph_seconds": round(build_s, 1), "graph": how,
            "qps": round(C3_NQ / gpu_s, 1), "note": "one host call (copies included), median of 3; launch "
                                                     "shapes autotuned on 4,096 other queries first",
            "autotune_s": round(tune_s, 1),
            "recall_at_10": round(hit / C3_NQ, 4),
            "reference_qps": round(C3_NQ / el, 1),
            "reference": f"search_batch per (filtered, k, ef) group ({len(batches)} calls), {threads} threads, "
                         f"simd {refcore.isa()}",
            "parity_vs_reference": {"queries": C3_NQ, "id_mismatches": ids, "distance_bit_mismatches": dist}}


# ---------------------------------------------------------------------------
# serving at 1M
# ---------------------------------------------------------------------------
SERVE_REQUESTS = 20_000
SERVE_LOADS = (0.25, 0.5, 0.75, 1.0)
SERVE_FILTERS = 16  # pool of distinct random 10%-density bitsets
SERVE_RECALL_REQUESTS = 2000
SERVE_PLAIN_REQUESTS = 500
SERVE_PARITY_REQUESTS = 1000  # requests also answered by the reference's search_batch
SERVE_FORMS = (
    # name, server options (batch slots and batch size: 4 x 8,192 queries
    # unless given; smaller batches trade peak for latency)
    ("fp32", dict(precision=0)),
    ("fp16_beam4_scan_8x2048", dict(precision=1, filter_scan=0.15, rerank_factor=4, lists_per_step=4,
                                    max_inflight=8, max_batch_queries=2048)),
    ("fp8_4warps_scan", dict(precision=2, filter_scan=0.15, rerank_factor=4, warps_per_query=4)),
    ("fp8_4warps_scan_8x2048", dict(precision=2, filter_scan=0.15, rerank_factor=4, warps_per_query=4,
                                    max_inflight=8, max_batch_queries=2048)),
    ("fp8_4warps_scan_15x256", dict(precision=2, filter_scan=0.15, rerank_factor=4, warps_per_query=4,
                                    max_inflight=15, max_batch_queries=256)),
)


def serving_workload():
    """Serving at 1M: 20,000 requests, log-uniform 1..256 queries each (seed 1
    mixture), k in {1,10,100}, ef in {16,32,..,512}, 20% with a bitset filter."""
    import workloads

    r = np.random.default_rng(4)
    nqs = np.minimum(np.floor(np.exp(r.uniform(0.0, np.log(257.0), SERVE_REQUESTS))), 256).astype(np.int64)
    ks = r.choice(np.array([1, 10, 100]), SERVE_REQUESTS)
    efs = r.choice(np.arange(16, 513, 16), SERVE_REQUESTS)
    fsel = np.where(r.random(SERVE_REQUESTS) < 0.2, r.integers(0, SERVE_FILTERS, SERVE_REQUESTS), -1)
    _, queries = workloads.int_mixture(1, HEAD_DIM, HEAD_CLUSTERS, int(nqs.sum()))
    rf = np.random.default_rng(5)
    masks = [rf.random(HEAD_N) < 0.1 for _ in range(SERVE_FILTERS)]
    return queries, nqs, ks, efs, fsel, masks


def run_serving(local, gpath):
    """The served, batched search at 1M (continuous batching): FP32 and the
    compressed forms, p50 / p99 / p999 at 25 / 50 / 75 / 100% of each form's
    peak, beside plain search_batch calls over the same queries."""
    import hnswgpu
    import workloads

    base, _ = head_workload()
    queries, nqs, ks, efs, fsel, masks = serving_workload()
    ix = hnswgpu.Index.load(gpath)
    ix.set_device(local)
    bitsets = [hnswgpu.Bitset(workloads.mask_to_words(m), HEAD_N) for m in masks]
    _, sample = workloads.int_mixture(1, HEAD_DIM, HEAD_CLUSTERS, 4096, qseed=2)
    sample_efs = np.random.default_rng(8).choice(np.arange(16, 513, 16), 4096).astype(np.uint32)
    t0 = time.time()
    for prec in (0, 2):
        ix.autotune(sample, k=10, ef_max=512, precision=prec, ef_per_query=sample_efs)
    tune_s = time.time() - t0
    offs = np.concatenate([[0], np.cumsum(nqs)])
    total_q = int(offs[-1])
    req_rows = np.repeat(np.arange(SERVE_REQUESTS), nqs)
    kq, efq, fq = ks[req_rows], efs[req_rows], fsel[req_rows]
    requests = [(queries[offs[i]:offs[i + 1]], int(ks[i]), int(efs[i]), bitsets[fsel[i]] if fsel[i] >= 0 else None)
                for i in range(SERVE_REQUESTS)]

    # plain FP32 search_batch, the reference's call: one call per request
    for i in range(50):
        ix.search_raw(*requests[i])
    t = time.perf_counter()
    for i in range(SERVE_PLAIN_REQUESTS):
        ix.search_raw(*requests[i])
    per_request_qps = int(offs[SERVE_PLAIN_REQUESTS]) / (time.perf_counter() - t)

    # batched FP32: all queries with per-query ef / k / filter in 65,536-query calls
    chunk = 65536
    plain = np.empty((total_q, 100), dtype=hnswgpu.NEIGHBOR)
    for rep in range(2):  # the first pass warms up
        t = time.perf_counter()
        for s in range(0, total_q, chunk):
            e = min(s + chunk, total_q)
            plain[s:e] = ix.search_batch_ex(queries[s:e], 100, ef_per_query=efq[s:e], k_per_query=kq[s:e],
                                            filters=bitsets, filter_of_query=fq[s:e]).reshape(e - s, 100)
        plain_s = time.perf_counter() - t
    plain_qps = total_q / plain_s

    # recall against exact k-NN over the first requests, per filter group
    sample_q = int(offs[SERVE_RECALL_REQUESTS])
    bf = hnswgpu.BruteForceIndex(HEAD_DIM, "l2")
    bf.add(base)
    gt = np.empty((sample_q, 100), dtype=np.int64)
    for f in range(-1, SERVE_FILTERS):
        sel = np.nonzero(fq[:sample_q] == f)[0]
        if sel.size:
            gt[sel] = bf.search_raw(queries[sel], 100, filter=masks[f] if f >= 0 else None)["label"]
    del bf

    def recall(labels_of_query):
        r_all, r10, n10 = 0.0, 0.0, 0
        for q in range(sample_q):
            k = int(kq[q])
            got = labels_of_query(q, k)
            r_all += len(np.intersect1d(got, gt[q, :k])) / k
            if k >= 10:
                r10 += len(np.intersect1d(got[:10], gt[q, :10])) / 10
                n10 += 1
        return round(r_all / sample_q, 4), round(r10 / max(n10, 1), 4)

    plain_recall = recall(lambda q, k: plain[q, :k]["label"].astype(np.int64))

    # the reference's own search_batch, one call per request (its k, ef and
    # filter), over the first requests: ids and distance bits against the
    # batched plain answers (and below against the served FP32 answers)
    import refcore

    rx = refcore.RefIndex(gpath)
    ref_bits = [refcore.Bitset(workloads.mask_to_words(m), HEAD_N) for m in masks]
    ref_rows = [rx.search_batch(requests[i][0], requests[i][1], requests[i][2], threads=0,
                                filt=ref_bits[fsel[i]] if fsel[i] >= 0 else None)
                for i in range(SERVE_PARITY_REQUESTS)]
    del rx

    def vs_reference(rows_of_request):
        ids = dist = 0
        for i in range(SERVE_PARITY_REQUESTS):
            got, ref = rows_of_request(i), ref_rows[i]
            ids += int((got["label"] != ref["label"]).any(1).sum())
            dist += int((got["distance"].view(np.uint32) != ref["distance"].view(np.uint32)).any(1).sum())
        return {"requests": SERVE_PARITY_REQUESTS, "queries": int(offs[SERVE_PARITY_REQUESTS]),
                "id_mismatches": ids, "distance_bit_mismatches": dist}
    out = {"workload": f"serving-L2-1M: the headline graph, {SERVE_REQUESTS} requests, {total_q} queries, 1..256 "
                       f"queries/request log-uniform, k in {{1,10,100}}, ef in {{16..512 step 16}}, 20% with a "
                       f"10%-density bitset (pool of {SERVE_FILTERS})",
           "autotune_s": round(tune_s, 1), "queries": total_q,
           "plain_fp32_search_batch_per_request": {
               "qps": round(per_request_qps, 1), "requests": SERVE_PLAIN_REQUESTS,
               "note": "one search_batch call per request (the reference API: one k / ef / filter per call)"},
           "batched_fp32_search_batch_ex": {"qps": round(plain_qps, 1), "recall_at_k": plain_recall[0],
                                            "recall_at_10": plain_recall[1], "queries_per_call": chunk,
                                            "parity_vs_reference": vs_reference(
                                                lambda i: plain[offs[i]:offs[i + 1], :ks[i]])}}
    for name, opts in SERVE_FORMS:
        srv = hnswgpu.Server(ix, **{"max_inflight": 4, "max_batch_queries": 8192, **opts})
        srv.replay(requests[:2000], np.zeros(2000))  # warm-up: encodes the copy, sizes the staging
        peak, outs = srv.replay(requests, np.zeros(SERVE_REQUESTS))
        same = all(np.array_equal(outs[i]["label"], plain[offs[i]:offs[i + 1], :ks[i]]["label"])
                   for i in range(SERVE_REQUESTS)) if opts["precision"] == 0 else None
        rec = recall(lambda q, k: outs[req_rows[q]][q - offs[req_rows[q]], :k]["label"].astype(np.int64))
        form = {"options": opts, "peak_qps": round(peak["qps"], 1), "recall_at_k": rec[0], "recall_at_10": rec[1],
                "peak_p50_ms": round(peak["p50_ms"], 3), "peak_mean_batch_queries": round(peak["mean_batch_queries"], 1),
                "loads": []}
        if same is not None:
            form["identical_to_plain_search_batch"] = bool(same)
            form["parity_vs_reference"] = vs_reference(lambda i: outs[i])
        mean_q = total_q / SERVE_REQUESTS
        for load in SERVE_LOADS:
            rate = load * peak["qps"] / mean_q  # requests per second
            arrivals = np.cumsum(np.random.default_rng(6).exponential(1.0 / rate, SERVE_REQUESTS))
            st, _ = srv.replay(requests, arrivals)
            form["loads"].append({"offered": load, "offered_qps": round(load * peak["qps"], 1),
                                  "qps": round(st["qps"], 1), "p50_ms": round(st["p50_ms"], 3),
                                  "p99_ms": round(st["p99_ms"], 3), "p999_ms": round(st["p999_ms"], 3),
                                  "mean_batch_queries": round(st["mean_batch_queries"], 1)})
        srv.close()
        out[name] = form
    best = max((n for n, o in SERVE_FORMS if o["precision"]), key=lambda n: out[n]["peak_qps"])
    out["served_compressed_form"] = best
    out["served_compressed_over_batched_fp32"] = round(out[best]["peak_qps"] / plain_qps, 3)
    out["served_compressed_over_served_fp32"] = round(out[best]["peak_qps"] / out["fp32"]["peak_qps"], 3)
    # the compressed form with the lowest p99 at half of its own peak
    half = {n: next(x for x in out[n]["loads"] if x["offered"] == 0.5) for n, o in SERVE_FORMS if o["precision"]}
    low = min(half, key=lambda n: half[n]["p99_ms"])
    out["lowest_p99_at_half_load"] = {"form": low, "p99_ms": half[low]["p99_ms"], "p50_ms": half[low]["p50_ms"],
                                      "peak_qps": out[low]["peak_qps"],
                                      "peak_over_batched_fp32": round(out[low]["peak_qps"] / plain_qps, 3)}
    return out


# ---------------------------------------------------------------------------
# precision at d = 960
# ---------------------------------------------------------------------------
PREC_N, PREC_DIM, PREC_NQ = 200_000, 960, 5_000
PREC_EFS = (40, 64, 128, 256, 512, 1024)
PREC_PARITY_EFS = (40, 128, 512)


def run_precision(local):
    """Precision path at d = 960: |N(0,1)| x per-dimension scale U[0.05, 1],
    200,000 rows, 5,000 queries.  For FP32, FP16 and FP8-E4M3 (per-row
    scale) traversal, each followed by the exact FP32 rerank: QPS (queries on
    the device, CUDA events, median of 3) and recall@10 per ef, the error of
    the returned distances against FP64, and the error of the compressed
    copies' traversal distances against FP64."""
    import torch

    import hnswgpu
    import workloads

    base, queries = workloads.scaled_abs_normal(PREC_N, PREC_DIM, PREC_NQ)
    gpath, build_s, how = bench_graph("l2-960", base)
    ix = hnswgpu.Index.load(gpath)
    ix.set_device(local)
    bf = hnswgpu.BruteForceIndex(PREC_DIM, "l2")
    bf.add(base)
    gt = bf.search_raw(queries, HEAD_K)["label"].astype(np.int64)
    del bf
    b64 = base.astype(np.float64)
    q64 = queries.astype(np.float64)
    # traversal distances of the compressed copies on a sample of (query, row) pairs
    rs = np.random.default_rng(7)
    pq = rs.integers(0, PREC_NQ, 20_000)
    px = rs.integers(0, PREC_N, 20_000)
    exact = ((b64[px] - q64[pq]) ** 2).sum(-1)
    x16 = base[px].astype(np.float16).astype(np.float64)
    xt = torch.from_numpy(base[px])
    sc = xt.abs().amax(1, keepdim=True) / 448.0
    sc = torch.where(sc > 0, sc, torch.ones_like(sc))
    x8 = ((xt / sc).to(torch.float8_e4m3fn).to(torch.float32) * sc).double().numpy()
    trav = {}
    for name, xx in (("fp16", x16), ("fp8_e4m3", x8)):
        rel = np.abs(((xx - q64[pq]) ** 2).sum(-1) - exact) / np.maximum(exact, 1e-30)
        trav[name] = {"mean_rel": float(rel.mean()), "max_rel": float(rel.max())}

    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    q_d = torch.from_numpy(queries).to(dev)
    out_d = torch.empty((PREC_NQ, HEAD_K, 4), dtype=torch.int32, device=dev)
    out = {"workload": f"precision-L2-960: n={PREC_N} d={PREC_DIM} M={M} efC={EFC} (reference add_batch), "
                       f"{PREC_NQ} queries, k={HEAD_K}",
           "graph_seconds": round(build_s, 1), "graph": how, "traversal_distance_error_vs_fp64": trav, "variants": {}}
    plain_rows = {}
    for name, prec in (("fp32", 0), ("fp16_rerank", 1), ("fp8_rerank", 2)):
        rows = []
        for ef in PREC_EFS:
            ms = []
            with torch.cuda.stream(stream):
                for i in range(5):
                    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    a.record(stream)
                    ix.search_device(q_d.data_ptr(), PREC_NQ, HEAD_K, ef, out_d.data_ptr(), stream.cuda_stream,
                                     precision=prec)
                    b.record(stream)
                    torch.cuda.synchronize()
                    if i >= 2:
                        ms.append(a.elapsed_time(b))
            rec = out_d.cpu().numpy().view(hnswgpu.NEIGHBOR).reshape(PREC_NQ, HEAD_K)
            got = rec["label"].astype(np.int64)
            d64 = ((b64[got] - q64[:, None, :]) ** 2).sum(-1)
            rel = np.abs(rec["distance"].astype(np.float64) - d64) / np.maximum(d64, 1e-30)
            if prec == 0 and ef in PREC_PARITY_EFS:
                plain_rows[ef] = rec.copy()
            rows.append({"ef": ef, "qps": round(PREC_NQ / (statistics.median(ms) / 1e3), 1),
                         "recall_at_10": round(workloads.recall_at_k(got, gt), 4),
                         "dist_mean_rel_err_vs_fp64": float(rel.mean()), "dist_max_rel_err_vs_fp64": float(rel.max())})
        out["variants"][name] = rows
    # the plain FP32 path against the reference's own search_batch on all
    # queries: ids and distance bits
    import refcore

    rx = refcore.RefIndex(gpath)
    out["fp32_parity_vs_reference"] = []
    for ef, rec in plain_rows.items():
        out["fp32_parity_vs_reference"].append({"ef": ef, "queries": PREC_NQ,
                                                **parity(rec, rx.search_batch(queries, HEAD_K, ef, threads=0))})
    del rx
    best = max(r["recall_at_10"] for r in out["variants"]["fp32"])
    out["recall_target_reached"] = best >= RECALL_TARGET
    out["largest_ef"] = PREC_EFS[-1]
    return out


# ---------------------------------------------------------------------------
# the reference arm
# ---------------------------------------------------------------------------
def run_reference(args, rank, world):
    """--impl reference: the reference's own Index::search_batch (its C++
    library compiled on this host) on the host cores, on the headline
    workload: the same graph file, the operating point picked the same way
    (smallest ef with recall@10 >= 0.95 on the first 10,000 queries, ground
    truth from the reference's brute force), each step one search_batch over
    20,000 queries of the batch with all host threads."""
    if rank != 0:
        return None
    try:
        import refcore

        refcore.lib()
    except Exception as e:  # noqa: BLE001
        return {"impl": "reference", "unavailable": f"the reference library could not be built here: {e}"[:300]}
    import workloads

    base, queries = head_workload()
    gpath, build_s, how = bench_graph("l2-1m", base)
    rx = refcore.RefIndex(gpath)
    threads = os.cpu_count() or 1
    sample = queries[:RECALL_SAMPLE]
    gt = refcore.bruteforce(base, sample, HEAD_K, threads=threads)["label"].astype(np.int64)
    rows = []
    for ef in HEAD_EFS:
        got = rx.search_batch(sample, HEAD_K, ef, threads=threads)["label"].astype(np.int64)
        rows.append({"ef": ef, "recall_at_10": round(workloads.recall_at_k(got, gt), 4)})
        if rows[-1]["recall_at_10"] >= RECALL_TARGET:
            break
    op = first_at_target(rows)
    ef = op["ef"]
    per = []
    for i in range(args.warmup + args.steps):
        s = (i * REF_STEP_QUERIES) % HEAD_NQ
        qs = queries[s:s + REF_STEP_QUERIES]
        t0 = time.perf_counter()
        rx.search_batch(qs, HEAD_K, ef, threads=threads)
        el = time.perf_counter() - t0
        if i >= args.warmup:
            per.append(el)
    v = REF_STEP_QUERIES * args.steps / sum(per)
    return {"metric": METRIC, "value": round(v, 1), "unit": "queries/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(sum(per) / args.steps * 1e3, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded 1,024-cluster integer Gaussian mixture, SIFT-1M shape)",
            "config": {"workload": WORKLOAD, "global_batch": REF_STEP_QUERIES, "form": "reference search_batch",
                       "ef": ef, "recall_at_10": op["recall_at_10"], "sweep": rows,
                       "graph": {"source": "reference add_batch (all host threads), FORMAT v1 file",
                                 "seconds": round(build_s, 1), "how": how}},
            "impl": "reference",
            "cpu_baseline": {"value": round(v, 1), "unit": "queries/s", "cores": threads, "kind": "reference",
                             "sample": f"{REF_STEP_QUERIES} queries of the batch per step, one search_batch call, "
                                       f"ef={ef}, {threads} threads, simd {refcore.isa()}, host {host_cpu()}"},
            "e2e": {"value": round(v, 1), "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-batched", action="store_true", help="skip the 200k mixed-ef block")
    ap.add_argument("--no-serving", action="store_true", help="skip the 1M serving block")
    ap.add_argument("--no-precision", action="store_true", help="skip the d=960 precision block")
    ap.add_argument("--no-build", action="store_true", help="skip the GPU graph-construction block")
    ap.add_argument("--launch", choices=["graph", "streams"], default="graph",
                    help="timed steps: one CUDA-graph replay, or kernel launches (for a profiler)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank, world, local = dist_env()
    if world > 1 and args.impl == "ours":
        import torch.distributed as dist

        dist.init_process_group("nccl")
    if args.impl == "reference":
        res = run_reference(args, rank, world)
    else:
        res = run_ours(args, rank, world, local)
    if rank == 0 and res is not None:
        print(json.dumps(res), flush=True)
    if world > 1 and args.impl == "ours":
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
