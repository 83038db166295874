/* hnswgpu_device.h -- the CUDA side of hnsw-gb300 behind a plain C ABI.
 *
 * This is the thin layer the C++20 host code (hnsw::Index) calls: it takes
 * the graph in the reference's in-memory layout as host pointers, mirrors it
 * into HBM once, and runs the batched query path as sm_103a kernels.  No C++
 * types, exceptions or STL cross this boundary: every call returns an
 * HGD_* status and hgd_last_error() describes the last failure on the calling
 * thread.
 *
 * Reference interfaces this layer replaces (paths within hnsw-engine):
 *   hgd_graph_upload      the arrays behind Index::Impl       src/index_impl.hpp:193-214
 *   hgd_graph_set_deleted the tombstone write of mark_deleted  src/index.cpp:308-318
 *   hgd_search            search_unlocked over a batch         src/search_layer.cpp:146-194
 *   hgd_bruteforce        BruteForceIndex::search_batch        src/brute_force.cpp:34-69
 *   hgd_build_graph       the linking half of add_batch        src/index.cpp:145-306
 */
#ifndef HNSWGPU_DEVICE_H
#define HNSWGPU_DEVICE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  HGD_OK = 0,
  HGD_EINVAL = 1,   /* bad argument (std::invalid_argument on the C++ side) */
  HGD_ERUNTIME = 2, /* runtime failure (std::runtime_error) */
  HGD_ECUDA = 3,    /* a CUDA call failed */
  HGD_ENOMEM = 4    /* device memory exhausted */
};

enum { HGD_METRIC_L2 = 0, HGD_METRIC_IP = 1, HGD_METRIC_COSINE = 2 };

/* Summation order of the distance reduction: the order of the reference's
 * kernel on the host whose results are to be reproduced bit for bit. */
enum { HGD_ORDER_SCALAR = 0, HGD_ORDER_AVX2 = 1, HGD_ORDER_AVX512 = 2, HGD_ORDER_NEON = 3 };

/* Traversal precision: FP32 is the reference's arithmetic; FP16 / FP8 (E4M3
 * with a per-vector scale) walk the graph on a compressed copy of the
 * vectors and rerank the final pool in exact FP32. */
enum { HGD_PREC_FP32 = 0, HGD_PREC_FP16 = 1, HGD_PREC_FP8 = 2 };

/* The exact scan that answers routed filtered queries (filter_scan_permille):
 * AUTO picks the one that reads fewer bytes; ALLOWED_ROWS reads only the rows
 * the query's filter allows, 8 queries per tensor-core tile (rows of <= 512
 * padded elements, a multiple of 128); EVERY_ROW is the tcgen05 GEMM over all
 * rows, 128 queries per tile, with the filter applied to its scores. */
enum { HGD_SCAN_AUTO = 0, HGD_SCAN_ALLOWED_ROWS = 1, HGD_SCAN_EVERY_ROW = 2 };

#define HGD_NCOUNTERS 8 /* per query: upper lists, upper distances, layer-0 lists,
                           layer-0 distances, visited, peak candidates, results,
                           tier flags (1 global visited set, 2 spill pool, 4 rerun) */

typedef struct hgd_graph hgd_graph;

/* A graph as Index::Impl holds it (FORMAT v1 sections + derived arrays). */
typedef struct {
  uint64_t count;
  uint64_t dim;
  uint64_t padded_dim;
  uint64_t M;
  int32_t metric;
  int32_t max_level;
  uint32_t entry_point;
  uint32_t reserved;
  const float* vectors;         /* count x padded_dim, prepared (cosine: unit) */
  const uint32_t* level0;       /* count x (1 + 2M): [n, ids...] */
  const uint32_t* upper;        /* upper_used words: per node, levels 1..L of [n, ids(M)] */
  uint64_t upper_used;
  const uint64_t* upper_offset; /* count, in uint32 units */
  const uint64_t* labels;       /* count */
  const uint8_t* levels;        /* count */
  const uint8_t* deleted;       /* count, 0/1 */
} hgd_graph_view;

/* A filter bitset: bit b of words[b >> 6].  label_space = 1: indexed by
 * external label (BitsetFilter); 0: indexed by internal id (already
 * translated on the host, e.g. a FunctionFilter).  Host memory. */
typedef struct {
  const uint64_t* words;
  uint64_t num_bits;
  int32_t label_space;
  int32_t reserved;
} hgd_bitset;

/* One batch.  Records of `out` are 16 bytes: {uint64 label, float distance,
 * uint32 zero}, the layout of hnsw::Neighbor; rows have stride k. */
typedef struct {
  const float* queries;          /* nq x dim, raw (cosine normalised on device) */
  int32_t queries_on_device;     /* 1: queries / ef / k arrays are device pointers */
  int32_t out_on_device;         /* 1: out / nres are device pointers */
  uint64_t nq;
  uint32_t k;                    /* row stride of out, >= every per-query k */
  uint32_t ef;                   /* 0: use ef_default */
  uint32_t ef_default;           /* the index's set_ef value */
  uint32_t precision;            /* HGD_PREC_* */
  const uint32_t* ef_per_query;  /* nullable; 0 entries mean ef_default */
  const uint32_t* k_per_query;   /* nullable */
  const hgd_bitset* filters;     /* host array of num_filters bitsets */
  uint32_t num_filters;
  uint32_t filter_scan_mode;     /* HGD_SCAN_*: the scan of routed queries (see filter_scan_permille) */
  const int32_t* filter_of_query; /* host, nq entries, -1 = unfiltered; NULL: filter 0 for all if any */
  void* out;                     /* nq*k records */
  uint32_t* nres;                /* nullable: per-query result count (no padding) */
  uint32_t* done_flags;          /* nullable, device-accessible (e.g. mapped pinned memory): entry q
                                    is set to 1 once query q's row of `out` is final */
  void* stream;                  /* cudaStream_t; NULL = the graph's stream */
  uint64_t* counters;            /* nullable host array, nq x HGD_NCOUNTERS */
  int32_t synchronize;           /* 1: return after the results are in `out`; 0: only enqueue on
                                    `stream` (host buffers must then be pinned and stay alive) */
  int32_t use_graph;             /* 1 (device-resident queries and out, no filters or counters,
                                    synchronize 0): the second call with the same pointers and
                                    shape captures the batch into a CUDA graph, later calls
                                    replay it */
  /* launch shape; 0 = chosen from ef (the autotuner's table) */
  uint32_t hash_slots;           /* visited hash per warp (power of two >= 256) */
  uint32_t cand_cap;             /* candidate head per warp (power of two >= 128) */
  uint32_t warps_per_block;      /* 1..4 */
  uint32_t pool_cap;             /* spill pool entries per warp before a rerun */
  /* FP16 / FP8 batches with host filters: queries whose filter allows at most
   * this many per mille of the nodes are answered by the exact tensor-core
   * scan over the allowed rows instead of a graph walk (0: off).  No
   * counterpart in the reference. */
  uint32_t filter_scan_permille;
  /* FP16 / FP8: the exact FP32 rerank covers the best rerank_factor x k
   * entries of the traversal pool (at least 32); 0 = the whole pool (ef
   * entries).  No counterpart in the reference. */
  uint32_t rerank_factor;
  /* FP16 / FP8 with dim <= 128: 4 = one CTA of four warps walks each query, a
   * beam search expanding four candidates per step (lower latency per query;
   * its visit order is not the reference's, recall is the bar); 0 or 1 = one
   * warp per query, the reference's order.  No counterpart in the reference. */
  uint32_t warps_per_query;
  /* FP16 / FP8 with dim <= 128 and one warp per query: 1..4 = a beam search
   * expanding this many neighbour lists per step, row distances on the
   * tensor cores (mma.sync m16n8k16), for throughput; 0 = the walk in the
   * reference's order.  No counterpart in the reference. */
  uint32_t lists_per_step;
} hgd_search_args;

int hgd_graph_upload(const hgd_graph_view* view, int device, int order, hgd_graph** out);

/* Streamed upload: the device graph built from FORMAT v1 sections as a
 * loader reads them, the host-to-device copies overlapped with the reads.
 * hgd_stream_begin takes the sizes of the view (count, dim, padded_dim, M,
 * metric, max_level, entry_point; its pointers are not read) and allocates
 * the device arrays and a ring of pinned staging buffers of chunk_bytes.
 * hgd_stream_buffer hands out the next staging buffer (after its previous
 * copy has ended); the loader fills it and passes it back with
 * hgd_stream_submit: section 0 (vectors), 1 (level0 in the file's layout) or
 * 2 (labels), at a byte offset into that section.  A buffer must not be
 * touched after its submit.  hgd_stream_finish takes the whole view (host
 * pointers, once the loader has validated the file), lays layer 0 out on the
 * device, builds the small parts and returns the graph; hgd_stream_abort
 * drops everything.  Every section 0-2 byte must be submitted exactly once. */
typedef struct hgd_stream hgd_stream;
int hgd_stream_begin(const hgd_graph_view* sizes, int device, int order, uint64_t chunk_bytes, hgd_stream** out);
int hgd_stream_buffer(hgd_stream* s, void** buf, uint64_t* cap);
int hgd_stream_submit(hgd_stream* s, int section, uint64_t offset, uint64_t bytes);
int hgd_stream_finish(hgd_stream* s, const hgd_graph_view* view, hgd_graph** out);
void hgd_stream_abort(hgd_stream* s);
int hgd_graph_set_deleted(hgd_graph* g, uint32_t id, int deleted);
int hgd_graph_set_order(hgd_graph* g, int order);
void hgd_graph_free(hgd_graph* g);
/* Device bytes held by the mirror (vectors, lists, labels, bitsets, scratch). */
uint64_t hgd_graph_device_bytes(const hgd_graph* g);

int hgd_search(hgd_graph* g, const hgd_search_args* a);

/* Launch shape of one ef bucket (bounds 16, 32, 64, 96, 128, 192, 256, 384,
 * 512, 768, 1024) for one precision, as chosen by the autotuner; a batch
 * without explicit shape fields uses the entry of each of its buckets.  No
 * counterpart in the reference. */
typedef struct {
  uint32_t precision;
  uint32_t ef_hi;
  uint32_t hash_slots;
  uint32_t cand_cap;
  uint32_t warps_per_block;
  uint32_t reserved;
} hgd_tune_entry;
int hgd_graph_set_tuning(hgd_graph* g, const hgd_tune_entry* entries, uint32_t n);
/* How a batch launches its ef buckets: HGD_LAUNCH_BUCKETS (one persistent
 * launch per bucket, concurrent on prioritised streams) or HGD_LAUNCH_SINGLE
 * (one persistent launch with the largest bucket's shape that drains every
 * query from a device queue, largest ef first).  Default BUCKETS. */
enum { HGD_LAUNCH_BUCKETS = 0, HGD_LAUNCH_SINGLE = 1 };
int hgd_graph_set_launch_mode(hgd_graph* g, int mode);
/* Bytes of per-warp shared memory of a shape (validation for tuners). */
uint32_t hgd_shape_smem_bytes(uint32_t hash_slots, uint32_t ef_hi, uint32_t cand_cap);
/* Device name and SM count of the graph's GPU. */
int hgd_graph_device_info(const hgd_graph* g, char* name, uint32_t name_cap, uint32_t* sms);

/* Exact k-NN over n prepared vectors (dim, unpadded), labels per row. */
typedef struct hgd_flat hgd_flat;
int hgd_flat_upload(const float* prepared, const uint64_t* labels, uint64_t n, uint64_t dim, int metric, int device,
                    int order, hgd_flat** out);
void hgd_flat_free(hgd_flat* f);
/* Which kernel answers hgd_bruteforce: HGD_BF_AUTO (the tensor-core GEMM
 * with exact rerank where the shape allows, else the CUDA-core scan),
 * HGD_BF_SCAN, or HGD_BF_TENSOR (HGD_EINVAL where unsupported).  No
 * counterpart in the reference, which has one CPU scan. */
enum { HGD_BF_AUTO = 0, HGD_BF_SCAN = 1, HGD_BF_TENSOR = 2 };
int hgd_flat_set_path(hgd_flat* f, int path);
/* The kernel that produced the last hgd_bruteforce answer (HGD_BF_SCAN or
 * HGD_BF_TENSOR; 0 before the first call). */
int hgd_flat_last_path(const hgd_flat* f);
int hgd_bruteforce(hgd_flat* f, const float* queries, uint64_t nq, uint32_t k, const hgd_bitset* filter, void* out,
                   void* stream);

/* Graph construction on the GPU: links nodes [first, count) into the graph
 * of nodes [0, first) -- the reference's Alg. 1 insertion with the Alg. 4
 * heuristic (src/index.cpp:127-241), in waves of new nodes that search the
 * graph built so far, one warp per node, with reverse edges merged per list
 * after each wave.  The host has stored the nodes already (rows prepared,
 * levels drawn, upper blocks placed: src/index.cpp:101-121); level0 and
 * upper are rewritten, and entry_point / max_level set, only when the call
 * succeeds (the lists come back into staging copies first).  The graph
 * is not the sequential build's (new nodes of one wave do not see each
 * other); it is judged on recall.  Limits: count < 2^24, 2 <= M <= 32,
 * padded_dim <= 1024, ef_construction <= 1024. */
typedef struct {
  uint64_t count;               /* nodes stored */
  uint64_t first;               /* first node to link */
  uint64_t dim, padded_dim, M, ef_construction;
  int32_t metric;               /* HGD_METRIC_* (cosine rows are unit vectors) */
  int32_t max_level;            /* in/out: top level of the graph (-1: empty) */
  uint32_t entry_point;         /* in/out: 0xFFFFFFFF for an empty graph */
  uint32_t wave_min;            /* smallest wave (0: 1) */
  uint32_t wave_max;            /* largest wave (0: four times the resident warps, sixteen with peers) */
  uint32_t waves;               /* out: waves launched */
  double wave_fraction;         /* new nodes per wave / nodes already linked (0: 0.02) */
  const float* vectors;         /* count x padded_dim (host) */
  uint32_t* level0;             /* count x (1 + 2M): [n, ids...] (host, in/out) */
  uint32_t* upper;              /* upper_words (host, in/out) */
  uint64_t upper_words;
  const uint64_t* upper_offset; /* count: word offset of a node's level-1 block */
  const uint8_t* levels;        /* count */
  uint64_t dropped_proposals;   /* out: reverse edges beyond a list's per-wave inbox (64) */
  int32_t peers;                /* 1: each new node re-chooses its list among its wave's nodes that
                                   chose the same neighbours (larger waves at equal recall) */
  int32_t reserved;
} hgd_build_args;
int hgd_build_graph(hgd_build_args* args, int device);

const char* hgd_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* HNSWGPU_DEVICE_H */
