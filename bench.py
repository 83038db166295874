"""Benchmark of the batched HNSW query path on GB300.

Workload (default): batched L2 at 200k -- n=200,000 vectors of d=128 from a
256-cluster integer Gaussian mixture (seed 0), M=16, ef_construction=200,
10,000 queries (seed 1) per step with per-query ef drawn uniformly from
{10,20,40,80,160,320}, k=10, answered in one persistent launch.  The data
are synthetic stand-ins with SIFT's shape (the ann-benchmarks sets are not
available offline); recall@10 is measured against exact k-NN.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  `value` is QPS with queries already in HBM
(device pointers, CUDA events on the launch stream, L2 flushed between
steps); `e2e` is QPS through the host C ABI with pinned host buffers, the
host->device copy of the queries and the device->host copy of the results
inside the timed region.  --impl reference times the reference algorithm on
the host cores (the oracle's C restatement of search_batch, all threads).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO / "hnsw-engine_gb300"))
sys.path.insert(0, str(REPO / "oracle"))

N_BASE, DIM, CLUSTERS, NQ, K = 200_000, 128, 256, 10_000, 10
EF_CHOICES = (10, 20, 40, 80, 160, 320)
# DRAM bytes of one search launch over this batch, read from an ncu capture
# (1.704 GB read + 0.432 GB written): below the algorithmic bytes, since part
# of the graph is served from L2
SEARCH_DRAM_BYTES = 2_136_463_000
SEARCH_L2_HIT_RATE = 0.509  # lts__t_sector_hit_rate of the same capture
M, EFC = 16, 200
METRIC = "QPS at recall@10≥0.95 (served/batched vs plain GPU, same GB300); p50/p99 ms"
WORKLOAD = "batched-L2-200k: n=200000 d=128 M=16 efC=200, 10000 queries/step, per-query ef U{10..320}, k=10"


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def workload(rank: int):
    import workloads

    base, queries = workloads.int_mixture(N_BASE, DIM, CLUSTERS, NQ)
    efs = np.random.default_rng(3 + rank).choice(np.array(EF_CHOICES, dtype=np.uint32), size=NQ)
    return base, queries, efs


def launches_per_batch(ef_max: int, single_launch: bool = False) -> int:
    """Kernels one batch enqueues: the ef-bucketing kernel, the query kernels
    (one largest-ef-first launch, or one per ef bucket 16, 32, 64, ... up to
    ef_max) and the rerun pass."""
    if single_launch:
        return 3
    buckets = 0
    for hi in (16, 32, 64, 96, 128, 192, 256, 384, 512, 768, 1024):
        if buckets == 11:
            break
        buckets += 1
        if hi >= ef_max:
            break
    else:
        buckets += 1
    return 2 + buckets


def algorithmic_bytes(cnt: np.ndarray) -> float:
    """Bytes a query must move: query row, upper/level-0 lists, one row per
    distance, the tombstone bit word per level-0 candidate, the output row."""
    row = 4 * 128
    up_list, l0_list = 4 * (1 + M), 4 * (1 + 2 * M)
    per_q = (4 * DIM + cnt[:, 0] * up_list + cnt[:, 1] * row + cnt[:, 2] * l0_list + cnt[:, 3] * row + K * 16)
    return float(per_q.sum())


class Clocks:
    """nvidia-smi samples during the timed region."""

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


def run_ours(args, rank, world, local):
    import torch

    import hnswgpu

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    base, queries, efs = workload(rank)
    # graph: built with the library's CPU add_batch (all host threads), saved in
    # FORMAT v1 and loaded back -- the file a CPU reference would also load
    tmp = Path(tempfile.mkdtemp(prefix="hnswbench"))
    gpath = tmp / "graph.idx"
    t0 = time.time()
    ix = hnswgpu.Index(DIM, "l2", M, EFC)
    ix.add(base, num_threads=0)
    ix.save(gpath)
    build_s = time.time() - t0
    ix = hnswgpu.Index.load(gpath)
    ix.set_device(local)

    # ground truth: exact k-NN on the GPU (brute force), FP32 exact on integer data
    bf = hnswgpu.BruteForceIndex(DIM, "l2")
    bf.add(base)
    gt = bf.search_raw(queries, K)["label"].astype(np.int64)
    del bf

    stream = torch.cuda.Stream(device=dev)
    q_d = torch.from_numpy(queries).to(dev)
    ef_d = torch.from_numpy(efs.astype(np.int32)).to(dev)
    out_d = torch.empty((NQ, K, 4), dtype=torch.int32, device=dev)  # 16-byte records
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # > L2 (129 MB)
    ef_max = int(efs.max())

    # launch shapes per ef bucket: autotuned on separate sample queries (seed 2)
    import workloads

    _, sample = workloads.int_mixture(N_BASE, DIM, CLUSTERS, NQ, qseed=2)
    sample_efs = np.random.default_rng(4).choice(np.array(EF_CHOICES, dtype=np.uint32), NQ)
    t0 = time.time()
    if args.tuning and Path(args.tuning).exists():
        # a table saved by an earlier run: the same launch shapes (a profiler
        # serialises the tuner's timed trials, so it would pick other shapes)
        tuning = json.loads(Path(args.tuning).read_text())
        ix.set_tuning(tuning)
    else:
        tuning = ix.autotune(sample, k=K, ef_max=int(efs.max()), precision=0, ef_per_query=sample_efs,
                             path=args.tuning)
    tune_s = time.time() - t0

    use_graph = args.launch == "graph"

    def step_device(graph=False):
        ix.search_device(q_d.data_ptr(), NQ, K, ef_max, out_d.data_ptr(), stream.cuda_stream, ef_ptr=ef_d.data_ptr(),
                         graph=graph)

    # recall and traversal counters of this batch (untimed; an NVTX range so a
    # profiler can pick these launches out)
    torch.cuda.nvtx.range_push("counters_batch")
    rec, cnt = ix.search_batch_ex(queries, K, ef_per_query=efs, counters=True)
    torch.cuda.nvtx.range_pop()
    got = rec["label"].astype(np.int64)

    recall = workloads.recall_at_k(got, gt)
    alg_bytes = algorithmic_bytes(cnt)

    # timed path: the batch's launch sequence replayed as one CUDA graph
    # (captured on the second warm-up step); the plain-stream path is timed
    # after it for comparison
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            flush.zero_()
            step_device(graph=use_graph)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        clocks = Clocks(local)
        with clocks:
            torch.cuda.nvtx.range_push("timed_steps")
            wall0 = time.perf_counter()
            for i in range(args.steps):
                flush.zero_()
                ev[i][0].record(stream)
                step_device(graph=use_graph)
                ev[i][1].record(stream)
            torch.cuda.synchronize()
            wall = time.perf_counter() - wall0
            torch.cuda.nvtx.range_pop()
        if world > 1:
            torch.distributed.barrier()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    dev_ms = sum(step_ms)
    # the same step launched kernel by kernel on forked streams
    stream_ms = []
    if use_graph:
        with torch.cuda.stream(stream):
            for i in range(args.warmup + args.steps):
                flush.zero_()
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                step_device(graph=False)
                b.record(stream)
                torch.cuda.synchronize()
                if i >= args.warmup:
                    stream_ms.append(a.elapsed_time(b))
    # device output equals the host-path output
    dev_rec = out_d.cpu().numpy().view(hnswgpu.NEIGHBOR).reshape(NQ, K)
    if not np.array_equal(dev_rec["label"], rec["label"]):
        raise RuntimeError("device-resident batch differs from the host-path batch")

    # e2e through the host C ABI with pinned host buffers
    q_pin = torch.from_numpy(queries).pin_memory()
    ef_pin = torch.from_numpy(efs.astype(np.uint32).view(np.int32)).pin_memory()
    out_pin = torch.empty((NQ, K, 4), dtype=torch.int32).pin_memory()
    qn = q_pin.numpy()
    efn = ef_pin.numpy().view(np.uint32)
    e2e_ms = []
    with torch.cuda.stream(stream):
        for i in range(args.warmup + args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            ix.search_batch_ex(qn, K, ef_per_query=efn, stream=stream.cuda_stream,
                               out=out_pin.numpy().view(hnswgpu.NEIGHBOR).reshape(-1))
            b.record(stream)
            torch.cuda.synchronize()
            if i >= args.warmup:
                e2e_ms.append(a.elapsed_time(b))
    e2e_total = sum(e2e_ms)

    if world > 1:  # the job's time is the slowest replica's
        import replicas

        dev_ms, e2e_total = replicas.max_over_ranks(dev_ms), replicas.max_over_ranks(e2e_total)
    qps = world * NQ * args.steps / (dev_ms / 1e3)
    e2e_qps = world * NQ * args.steps / (e2e_total / 1e3)
    per_launch_ms = dev_ms / args.steps
    peak, peak_kind = measured_peaks()
    achieved = alg_bytes / (per_launch_ms / 1e3) / 1e9
    result = {
        "metric": METRIC, "value": round(qps, 1), "unit": "queries/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(per_launch_ms, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded Gaussian mixture, SIFT shape)",
        "config": {"workload": WORKLOAD, "global_batch": world * NQ, "recall_at_10": round(recall, 4),
                   "ef_mix": list(EF_CHOICES), "l2_flush": "256 MiB write before every timed step",
                   "parallelism": f"replicas x{world} (queries per replica fixed)", "build_s": round(build_s, 2),
                   "launch": ("one CUDA-graph replay per step" if use_graph else "kernel launches per step") +
                             (" (bucket kernel, one persistent largest-ef-first search launch, rerun pass)"
                              if tuning["launch_mode"] == 1 else
                              " (bucket kernel, per-ef-bucket persistent launches on prioritised forked streams, "
                              "rerun pass)"),
                   "streams_ms_per_step": round(statistics.median(stream_ms), 4) if stream_ms else None,
                   "autotune": {"seconds": round(tune_s, 2),
                                "sample": f"{NQ} seed-2 queries of the same mixture, ef from the same set (seed 4)",
                                "launch_mode": ["per-bucket launches", "one largest-ef-first launch"][tuning["launch_mode"]],
                                "buckets": {str(e["ef_hi"]): [e["hash_slots"], e["cand_cap"], e["warps_per_block"],
                                                              round(e["default_us_per_query"] / max(e["us_per_query"], 1e-9), 3)]
                                            for e in tuning["entries"]},
                                "fields": "hash_slots, cand_cap, warps_per_block (0 = default), speed-up over default"},
                   "mean_l0_expansions": round(float(cnt[:, 2].mean()), 2),
                   "mean_l0_distances": round(float(cnt[:, 3].mean()), 2)},
        "e2e": {"value": round(e2e_qps, 1), "unit": "queries/s", "h2d_bytes_per_step": int(NQ * DIM * 4 + NQ * 4),
                "d2h_bytes_per_step": int(NQ * K * 16)},
        "gpu_launches": launches_per_batch(ef_max, tuning["launch_mode"] == 1) * args.steps,
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": SEARCH_DRAM_BYTES,
                     "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of this workload's "
                                       "search launch (one batch, cold L2)",
                     "l2_hit_rate": SEARCH_L2_HIT_RATE,
                     "peak_source": peak_kind, "algorithmic_bytes_per_launch": int(alg_bytes)},
        "clocks": clocks.summary(),
        "wall_s": round(wall, 3),
    }
    if rank == 0 and world == 1:
        result["cpu_baseline"] = cpu_baseline(gpath, queries, efs)
        del ix
        if not args.no_serving:
            result["serving"] = run_serving(local)
        if not args.no_precision:
            result["precision"] = run_precision(local)
    return result


SERVE_N, SERVE_CLUSTERS, SERVE_REQUESTS = 1_000_000, 1024, 20_000
SERVE_LOADS = (0.25, 0.5, 0.75, 1.0)
SERVE_FILTERS = 16  # pool of distinct random 10%-density bitsets
SERVE_RECALL_REQUESTS = 2000
SERVE_PLAIN_REQUESTS = 2000
SERVE_RERANK_FACTOR = 4  # FP8 forms: exact rerank of the pool's best 4 x k (at least 32)


def serving_workload():
    """Serving at 1M: 20,000 requests, log-uniform 1..256 queries each (seed 1
    mixture), k in {1,10,100}, ef in {16,32,..,512}, 20% with a bitset filter."""
    import workloads

    r = np.random.default_rng(4)
    nqs = np.minimum(np.floor(np.exp(r.uniform(0.0, np.log(257.0), SERVE_REQUESTS))), 256).astype(np.int64)
    ks = r.choice(np.array([1, 10, 100]), SERVE_REQUESTS)
    efs = r.choice(np.arange(16, 513, 16), SERVE_REQUESTS)
    fsel = np.where(r.random(SERVE_REQUESTS) < 0.2, r.integers(0, SERVE_FILTERS, SERVE_REQUESTS), -1)
    base, queries = workloads.int_mixture(SERVE_N, DIM, SERVE_CLUSTERS, int(nqs.sum()))
    rf = np.random.default_rng(5)
    masks = [rf.random(SERVE_N) < 0.1 for _ in range(SERVE_FILTERS)]
    return base, queries, nqs, ks, efs, fsel, masks


def run_serving(local):
    """The served, batched search at 1M (FP8-E4M3 traversal + exact FP32 rerank,
    and plain FP32) next to one plain FP32 search_batch over the same queries."""
    import hnswgpu
    import workloads

    base, queries, nqs, ks, efs, fsel, masks = serving_workload()
    t0 = time.time()
    ix = hnswgpu.Index(DIM, "l2", M, EFC)
    ix.add(base, num_threads=0)
    build_s = time.time() - t0
    ix.set_device(local)
    bitsets = [hnswgpu.Bitset(workloads.mask_to_words(m), SERVE_N) for m in masks]
    # launch shapes for both forms, tuned on separate queries (seed 2, same
    # cluster centres) with the serving ef mix
    _, sample = workloads.int_mixture(1, DIM, SERVE_CLUSTERS, 4096, qseed=2)
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

    # plain FP32 search_batch, the reference's call: one call per request (its
    # own k, ef and filter), one after another, on a sample of the requests
    for i in range(200):
        ix.search_raw(*requests[i])
    t = time.perf_counter()
    for i in range(SERVE_PLAIN_REQUESTS):
        ix.search_raw(*requests[i])
    per_request_s = time.perf_counter() - t
    per_request_qps = int(offs[SERVE_PLAIN_REQUESTS]) / per_request_s

    # batched FP32: all queries with per-query ef / k / filter in 65,536-query
    # calls (host buffers in and out)
    chunk = 65536
    plain = np.empty((total_q, 100), dtype=hnswgpu.NEIGHBOR)
    for rep in range(2):  # the first pass mirrors the graph and warms up
        t = time.perf_counter()
        for s in range(0, total_q, chunk):
            e = min(s + chunk, total_q)
            plain[s:e] = ix.search_batch_ex(queries[s:e], 100, ef_per_query=efq[s:e], k_per_query=kq[s:e],
                                            filters=bitsets, filter_of_query=fq[s:e]).reshape(e - s, 100)
        plain_s = time.perf_counter() - t
    plain_qps = total_q / plain_s

    # recall against exact k-NN (brute force on the GPU, exact on integer data)
    # over the first requests, per filter group
    sample_q = int(offs[SERVE_RECALL_REQUESTS])
    bf = hnswgpu.BruteForceIndex(DIM, "l2")
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
    out = {"workload": f"serving-L2-1M: n={SERVE_N} d={DIM} M={M} efC={EFC}, {SERVE_REQUESTS} requests, "
                       f"{total_q} queries, 1..256 queries/request log-uniform, k in {{1,10,100}}, "
                       f"ef in {{16..512 step 16}}, 20% with a 10%-density bitset (pool of {SERVE_FILTERS})",
           "build_s": round(build_s, 1), "autotune_s": round(tune_s, 1), "queries": total_q,
           "plain_fp32_search_batch_per_request": {
               "qps": round(per_request_qps, 1), "requests": SERVE_PLAIN_REQUESTS,
               "note": "one search_batch call per request (the reference API: one k / ef / filter per call)"},
           "batched_fp32_search_batch_ex": {"qps": round(plain_qps, 1), "recall_at_k": plain_recall[0],
                                            "recall_at_10": plain_recall[1], "queries_per_call": chunk}}
    # forms: FP32 walk; FP8 walk + exact rerank of the pool's best
    # SERVE_RERANK_FACTOR x k; the same with requests whose
    # filter allows <= 15% of the nodes answered by the exact tensor-core
    # scan; the last also walks with four warps per query (beam search)
    for name, prec, scan, rf, wpq in (("fp32", 0, 0.0, 0, 1), ("fp8_rerank", 2, 0.0, SERVE_RERANK_FACTOR, 1),
                                      ("fp8_rerank_filter_scan", 2, 0.15, SERVE_RERANK_FACTOR, 1),
                                      ("fp8_rerank_filter_scan_4warps", 2, 0.15, SERVE_RERANK_FACTOR, 4)):
        srv = hnswgpu.Server(ix, max_inflight=4, max_batch_queries=8192, precision=prec, filter_scan=scan,
                             rerank_factor=rf, warps_per_query=wpq)
        srv.replay(requests[:2000], np.zeros(2000))  # warm-up: encodes the FP8 copy, sizes the staging
        peak, outs = srv.replay(requests, np.zeros(SERVE_REQUESTS))
        same = all(np.array_equal(outs[i]["label"], plain[offs[i]:offs[i + 1], :ks[i]]["label"])
                   for i in range(SERVE_REQUESTS)) if prec == 0 else None
        rec = recall(lambda q, k: outs[req_rows[q]][q - offs[req_rows[q]], :k]["label"].astype(np.int64))
        form = {"peak_qps": round(peak["qps"], 1), "recall_at_k": rec[0], "recall_at_10": rec[1],
                "rerank_factor": rf, "warps_per_query": wpq,
                "peak_p50_ms": round(peak["p50_ms"], 3), "peak_mean_batch_queries": round(peak["mean_batch_queries"], 1),
                "loads": []}
        if same is not None:
            form["identical_to_plain_search_batch"] = bool(same)
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
    best = max(("fp8_rerank", "fp8_rerank_filter_scan", "fp8_rerank_filter_scan_4warps"),
               key=lambda f: out[f]["peak_qps"])
    out["served_fp8_form"] = best
    out["served_fp8_over_plain_fp32"] = round(out[best]["peak_qps"] / per_request_qps, 3)
    out["served_fp8_over_batched_fp32"] = round(out[best]["peak_qps"] / plain_qps, 3)
    return out


PREC_N, PREC_DIM, PREC_NQ = 200_000, 960, 5_000
PREC_EFS = (40, 64, 128, 256, 512)


def run_precision(local):
    """Precision path at d=960: |N(0,1)| x per-dimension scale U[0.05, 1],
    200,000 rows, 5,000 queries.  For FP32, FP16 and FP8-E4M3 (per-row scale)
    traversal, each followed by the exact FP32 rerank: QPS and recall@10 per
    ef, the error of the returned distances against FP64, and the error of
    the compressed copies' traversal distances against FP64."""
    import torch

    import hnswgpu
    import workloads

    base, queries = workloads.scaled_abs_normal(PREC_N, PREC_DIM, PREC_NQ)
    t0 = time.time()
    ix = hnswgpu.Index(PREC_DIM, "l2", M, EFC)
    ix.add(base, num_threads=0)
    build_s = time.time() - t0
    ix.set_device(local)
    bf = hnswgpu.BruteForceIndex(PREC_DIM, "l2")
    bf.add(base)
    gt = bf.search_raw(queries, K)["label"].astype(np.int64)
    del bf
    b64 = base.astype(np.float64)
    q64 = queries.astype(np.float64)

    def fp64_dist(qi, ids):
        return ((b64[ids] - q64[qi][:, None, :]) ** 2).sum(-1)

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

    out = {"workload": f"precision-L2-960: n={PREC_N} d={PREC_DIM} M={M} efC={EFC}, {PREC_NQ} queries, k={K}",
           "build_s": round(build_s, 1), "traversal_distance_error_vs_fp64": trav, "variants": {}}
    for name, prec in (("fp32", 0), ("fp16_rerank", 1), ("fp8_rerank", 2)):
        rows = []
        for ef in PREC_EFS:
            ix.search_batch_ex(queries[:256], K, ef, precision=prec)  # warm-up (builds the copy once)
            t = time.perf_counter()
            rec = ix.search_batch_ex(queries, K, ef, precision=prec)
            el = time.perf_counter() - t
            got = rec["label"].astype(np.int64)
            d64 = fp64_dist(np.arange(PREC_NQ), got)
            rel = np.abs(rec["distance"].astype(np.float64) - d64) / np.maximum(d64, 1e-30)
            rows.append({"ef": ef, "qps": round(PREC_NQ / el, 1), "recall_at_10": round(workloads.recall_at_k(got, gt), 4),
                         "dist_mean_rel_err_vs_fp64": float(rel.mean()), "dist_max_rel_err_vs_fp64": float(rel.max())})
        out["variants"][name] = rows
    return out


def cpu_baseline(gpath, queries, efs, sample=None):
    """The reference algorithm (oracle restatement of search_batch) on the host
    cores, grouped per ef like one reference call per group."""
    import pyoracle

    threads = os.cpu_count() or 1
    ox = pyoracle.OracleIndex(gpath, isa=pyoracle.host_isa())
    nq = queries.shape[0] if sample is None else sample
    qs, es = queries[:nq], efs[:nq]
    t0 = time.perf_counter()
    for ef in EF_CHOICES:
        sel = es == ef
        if sel.any():
            ox.search_batch(qs[sel], K, int(ef), threads=threads)
    el = time.perf_counter() - t0
    return {"value": round(nq / el, 1), "unit": "queries/s", "cores": threads, "kind": "port",
            "sample": f"{nq} queries of the same mixed-ef batch, one search_batch per ef group, "
                      f"{threads} threads, distance order {pyoracle.host_isa()}"}


def run_reference(args, rank, world):
    """--impl reference: the reference algorithm on the host cores."""
    if rank != 0:
        return None
    import hnswgpu  # only to build the same graph file

    base, queries, efs = workload(0)
    tmp = Path(tempfile.mkdtemp(prefix="hnswref"))
    gpath = tmp / "graph.idx"
    ix = hnswgpu.Index(DIM, "l2", M, EFC)
    ix.add(base, num_threads=0)
    ix.save(gpath)
    sample = 4000
    vals = []
    for i in range(args.warmup + args.steps):
        r = cpu_baseline(gpath, queries, efs, sample=sample)
        if i >= args.warmup:
            vals.append(r["value"])
    v = statistics.median(vals)
    ms = sample / v * 1e3
    return {"metric": METRIC, "value": round(v, 1), "unit": "queries/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded Gaussian mixture, SIFT shape)",
            "config": {"workload": WORKLOAD}, "impl": "reference",
            "cpu_baseline": {"value": round(v, 1), "unit": "queries/s", "cores": os.cpu_count(), "kind": "port",
                             "sample": f"{sample} queries per step of the mixed-ef batch, all host threads"},
            "e2e": {"value": round(v, 1), "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-serving", action="store_true", help="skip the 1M serving measurement")
    ap.add_argument("--no-precision", action="store_true", help="skip the d=960 precision measurement")
    ap.add_argument("--tuning", default=None,
                    help="launch-shape table: loaded if the file exists, else autotuned and saved there")
    ap.add_argument("--launch", choices=["graph", "streams"], default="graph",
                    help="timed step: one CUDA-graph replay, or kernel launches on forked streams")
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
