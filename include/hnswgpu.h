/* hnswgpu.h -- C ABI of hnsw-gb300 for foreign-function callers.
 *
 * Each entry point is one hnsw::Index operation (GPU-answered queries, CPU
 * construction, FORMAT v1 files), with plain pointers and sizes and an
 * integer status instead of exceptions: HG_OK, or HG_EINVAL where the
 * reference throws std::invalid_argument, HG_ERANGE for std::out_of_range,
 * HG_ERUNTIME for std::runtime_error (I/O, corrupt file, read-only, full,
 * CUDA failure).  hg_last_error() returns the message of the last failure on
 * the calling thread.
 *
 * Reference interface each entry point replaces (paths within hnsw-engine):
 *   hg_index_create        Index(const Params&)                 include/hnsw/index.hpp:39; src/index.cpp:48-67
 *   hg_index_load          Index::load(path, mmap)              include/hnsw/index.hpp:86; src/persist.cpp:476-541
 *   hg_index_load_device   Index::load with the device graph built while the file is read (no counterpart)
 *   hg_index_save          Index::save                          include/hnsw/index.hpp:83; src/persist.cpp:421-474
 *   hg_index_free          ~Index                               include/hnsw/index.hpp:40
 *   hg_index_add_batch     Index::add_batch                     include/hnsw/index.hpp:50; src/index.cpp:273-306
 *   hg_index_add_batch_gpu Index::add_batch with the linking on the GPU  src/index.cpp:145-306 (no counterpart call)
 *   hg_index_search        Index::search                        include/hnsw/index.hpp:55; src/search_layer.cpp:173-178
 *   hg_index_search_batch  Index::search_batch                  include/hnsw/index.hpp:59; src/search_layer.cpp:180-194
 *   hg_index_search_batch_ex  search_batch with per-query ef/k/filter (one reference call per group)
 *   hg_index_mark_deleted  Index::mark_deleted                  include/hnsw/index.hpp:64; src/index.cpp:308-318
 *   hg_index_is_deleted / hg_index_contains / hg_index_get_vector / accessors
 *                          include/hnsw/index.hpp:65-81;  src/index.cpp:320-379
 *   hg_index_set_ef        Index::set_ef                        src/index.cpp:352-356
 *   hg_bruteforce_*        BruteForceIndex                      include/hnsw/index.hpp:103-118; src/brute_force.cpp
 *   hg_set_distance_order  simd::set_active                     include/hnsw/metric.hpp:212
 * Filters: hg_filter describes a BitsetFilter (label bitset) or a
 * FunctionFilter (a predicate callback), include/hnsw/filter.hpp:12-48.
 */
#ifndef HNSWGPU_H
#define HNSWGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { HG_OK = 0, HG_EINVAL = 1, HG_ERUNTIME = 2, HG_ERANGE = 3 };
enum { HG_METRIC_L2 = 0, HG_METRIC_IP = 1, HG_METRIC_COSINE = 2 };
enum { HG_ORDER_SCALAR = 0, HG_ORDER_AVX2 = 1, HG_ORDER_AVX512 = 2, HG_ORDER_NEON = 3 };
enum { HG_FILTER_NONE = 0, HG_FILTER_BITSET = 1, HG_FILTER_PREDICATE = 2 };
/* The exact scan of routed filtered queries: AUTO = the one that reads fewer
 * bytes; ALLOWED_ROWS = only the rows the filter allows (tensor-core tiles
 * of 8 queries; padded row width a multiple of 128, at most 512); EVERY_ROW
 * = the tcgen05 GEMM over all rows (tiles of 128 queries). */
enum { HG_SCAN_AUTO = 0, HG_SCAN_ALLOWED_ROWS = 1, HG_SCAN_EVERY_ROW = 2 };

#define HG_INVALID_LABEL (~(uint64_t)0)

typedef struct hg_index hg_index;
typedef struct hg_bruteforce hg_bruteforce;

/* Layout of hnsw::Neighbor: 16 bytes, the last 4 are zero. */
typedef struct {
  uint64_t label;
  float distance;
  uint32_t reserved;
} hg_neighbor;

/* A label filter.  BITSET: bit l of words[l / 64] allows label l, labels >=
 * num_labels are rejected.  PREDICATE: fn(label, ctx) != 0 allows label; it
 * is called once per node of the index before the GPU search starts. */
typedef struct {
  int32_t kind;
  int32_t reserved;
  const uint64_t* words;
  uint64_t num_labels;
  int (*fn)(uint64_t label, void* ctx);
  void* ctx;
} hg_filter;

/* Optional batch controls (hnsw::SearchOptions). */
typedef struct {
  const uint32_t* ef_per_query;    /* nq entries or NULL */
  const uint32_t* k_per_query;     /* nq entries (each 1..k) or NULL */
  const hg_filter* filters;        /* filter table */
  size_t num_filters;
  const int32_t* filter_of_query;  /* nq entries, -1 = none; NULL = filter 0 for all */
  void* stream;                    /* cudaStream_t, NULL = the index's own */
  int32_t precision;               /* 0 fp32; 1 fp16; 2 fp8 traversal with exact fp32 rerank */
  int32_t use_graph;               /* 1 with device-resident queries and out (no filters or
                                      counters): the batch is captured into a CUDA graph on its
                                      second call with the same pointers and shape, then replayed */
  uint64_t* counters;              /* nq x 8 traversal counters or NULL */
  uint32_t hash_slots;             /* launch shape, 0 = automatic: visited-hash slots per warp */
  uint32_t cand_cap;               /* candidate head capacity per warp */
  uint32_t warps_per_block;
  uint32_t pool_cap;               /* spill-pool entries per warp before a query is rerun */
  int32_t queries_on_device;       /* 1: qs, ef_per_query, k_per_query are device pointers
                                      (then ef must bound every per-query ef) */
  int32_t out_on_device;           /* 1: out is a device pointer; the call returns once the
                                      work is queued on `stream` */
  uint32_t filter_scan_permille;   /* precision 1 / 2: queries whose filter allows at most this
                                      many per mille of the nodes are answered by the exact
                                      tensor-core scan over the allowed rows (0: off) */
  uint32_t rerank_factor;          /* precision 1 / 2: exact rerank of the best rerank_factor x k
                                      pool entries (at least 32); 0 = the whole pool */
  uint32_t warps_per_query;        /* precision 1 / 2, dim <= 128: 4 = four warps walk each query
                                      (beam search, lower latency); 0 / 1 = one warp */
  uint32_t lists_per_step;         /* precision 1 / 2, dim <= 128, warps_per_query <= 1: 1..4 = one
                                      warp walks each query as a beam search expanding this many
                                      lists per step, distances on the tensor cores; 0 = the
                                      one-warp walk in the reference's order */
  uint32_t filter_scan_mode;       /* HG_SCAN_*: the exact scan of routed queries */
  uint32_t reserved;
} hg_batch_options;

const char* hg_last_error(void);

int hg_index_create(size_t dim, int metric, size_t M, size_t ef_construction, size_t max_elements, uint64_t seed,
                    hg_index** out);
int hg_index_load(const char* path, int mmap, hg_index** out);
/* hg_index_load, and the graph mirrored to `device` in the same pass: the
 * vectors, layer 0 and labels go to the device through pinned staging
 * buffers as they are read and hashed.  Same validation and errors. */
int hg_index_load_device(const char* path, int mmap, int device, hg_index** out);
int hg_index_save(const hg_index* idx, const char* path);
void hg_index_free(hg_index* idx);
int hg_index_add_batch(hg_index* idx, const float* vecs, const uint64_t* labels, size_t n, size_t num_threads);

/* add_batch with the graph linking on the GPU (no counterpart in the
 * reference).  The same validation, errors, stored rows, labels and levels
 * as hg_index_add_batch; new nodes are linked in waves that search the graph
 * built so far, one warp per node, with the reverse edges merged per list
 * after each wave.  The graph is not the CPU build's (as a threaded build's
 * is not); it is judged on recall.  Limits: size + n < 2^24, M <= 32,
 * dim <= 1024, ef_construction <= 1024 (HG_EINVAL beyond them).  opt may be
 * NULL; its out fields report the waves and the reverse edges dropped. */
typedef struct {
  int32_t device;              /* CUDA device, -1 = the index's */
  uint32_t wave_min;           /* smallest wave, 0 = 1 */
  uint32_t wave_max;           /* largest wave, 0 = four (peers: sixteen) times the resident warps */
  uint32_t waves;              /* out */
  double wave_fraction;        /* new nodes per wave / nodes already linked, 0 = 0.02 */
  uint64_t dropped_proposals;  /* out */
  double seconds;              /* out: wall time of the GPU linking */
  int32_t peers;               /* 1: each new node re-chooses its list among its wave's nodes that
                                  chose the same neighbours (larger waves at equal recall) */
  int32_t reserved;
} hg_build_options;
int hg_index_add_batch_gpu(hg_index* idx, const float* vecs, const uint64_t* labels, size_t n,
                           hg_build_options* opt);

int hg_index_search(const hg_index* idx, const float* q, size_t k, size_t ef, const hg_filter* filter,
                    hg_neighbor* out, size_t* n_out);
int hg_index_search_batch(const hg_index* idx, const float* qs, size_t nq, size_t k, size_t ef, hg_neighbor* out,
                          size_t num_threads, const hg_filter* filter);
int hg_index_search_batch_ex(const hg_index* idx, const float* qs, size_t nq, size_t k, size_t ef,
                             hg_neighbor* out, const hg_batch_options* opt);

/* Launch-shape autotuner (no counterpart in the reference): times the query
 * kernel's candidate shapes per ef bucket (up to ef_max) on `qs` (nq sample
 * queries, host memory), installs the fastest for `precision` and writes the
 * table as JSON into json (capacity json_cap; *json_len = bytes needed).
 * With ef_per_query (host, nq entries) the sample runs as one mixed batch and
 * the shapes are chosen on its total time.  hg_index_set_tuning installs a
 * table written earlier. */
int hg_index_autotune(hg_index* idx, const float* qs, size_t nq, size_t k, size_t ef_max, int precision,
                      const uint32_t* ef_per_query, char* json, size_t json_cap, size_t* json_len);
int hg_index_set_tuning(hg_index* idx, const char* json);

int hg_index_mark_deleted(hg_index* idx, uint64_t label);
int hg_index_is_deleted(const hg_index* idx, uint64_t label, int* out);
int hg_index_contains(const hg_index* idx, uint64_t label, int* out);
int hg_index_get_vector(const hg_index* idx, uint64_t label, float* out, size_t dim);
int hg_index_set_ef(hg_index* idx, size_t ef);
int hg_index_set_device(hg_index* idx, int device);

size_t hg_index_size(const hg_index* idx);
size_t hg_index_dim(const hg_index* idx);
int hg_index_metric(const hg_index* idx);
size_t hg_index_M(const hg_index* idx);
size_t hg_index_ef_construction(const hg_index* idx);
size_t hg_index_ef(const hg_index* idx);
size_t hg_index_capacity(const hg_index* idx);
int hg_index_max_level(const hg_index* idx);
int hg_index_read_only(const hg_index* idx);
size_t hg_index_memory_usage(const hg_index* idx);

int hg_bruteforce_create(size_t dim, int metric, hg_bruteforce** out);
int hg_bruteforce_add(hg_bruteforce* bf, const float* vecs, const uint64_t* labels, size_t n);
int hg_bruteforce_search_batch(const hg_bruteforce* bf, const float* qs, size_t nq, size_t k, hg_neighbor* out,
                               const hg_filter* filter);
void hg_bruteforce_free(hg_bruteforce* bf);
/* GPU kernel choice for brute force: 0 auto, 1 CUDA-core scan, 2 tensor-core
 * GEMM with exact rerank; and the kernel that answered the last search.  No
 * counterpart in the reference. */
int hg_bruteforce_set_path(hg_bruteforce* bf, int path);
int hg_bruteforce_last_path(const hg_bruteforce* bf);

/* A batch that allocates nothing on the device.  For callers that cannot
 * call cudaMalloc while they search -- a serving process that runs next to
 * other GPU work under a fixed memory budget, code inside a region where an
 * allocation would synchronise the device or is not permitted, a framework
 * that owns every device allocation.  Queries (nq x dim float32) and out
 * (nq x k hg_neighbor records) are device pointers the caller allocated; one
 * ef for the batch (0 = the index's set_ef value); no filter (tombstones
 * apply).  The work is enqueued on `stream` (NULL = the index's stream) and
 * the call returns without synchronising.  Scratch lives in a static device
 * array of about 15.4 MiB that every GPU using the library holds until exit;
 * batches that overlap on the GPU share it and race, so issue them on one
 * stream or serialise them.  The first call on a device looks up that
 * array's device address; make it before any stream capture.  The graph must
 * already be mirrored on the GPU (any earlier allocating search does it).
 * Limits: nq <= 65536, index size <= 2^20 nodes, max(ef, k) <= 512; larger
 * requests return HG_EINVAL.  Cost: the walk runs on a fixed 48 warps (12
 * blocks of 4) whatever the GPU, so a large batch takes several times as
 * long as through the allocating calls, and queries that outgrow its
 * 2,048-key spill pool are finished one after another by a single warp.
 * The array's device address is looked up once per device and kept: a
 * device reset after the first call is not supported.  No counterpart in
 * the reference. */
int hg_index_search_batch_noalloc(const hg_index* idx, const float* queries, size_t nq, size_t k, size_t ef,
                                  hg_neighbor* out, void* stream);

/* Continuous-batching server over one index (an addition; the reference has
 * no serving loop).  Requests -- a block of queries with their own k, ef and
 * optional filter -- are queued and admitted into GPU batches as batch slots
 * and the device-memory budget allow; batches in flight overlap on the GPU.
 * A request's results do not depend on the requests it is batched with.
 * The query, output and filter memory of a request must stay valid until
 * hg_server_wait returns for it (or hg_server_replay returns). */
typedef struct hg_server hg_server;
typedef struct {
  uint32_t max_inflight;       /* batches on the GPU at once (1..15, default 4) */
  uint32_t max_batch_queries;  /* queries admitted into one batch (default 4096) */
  uint64_t memory_budget;      /* device bytes for batches in flight; 0 = half the free memory */
  int32_t precision;           /* 0 fp32; 1 fp16; 2 fp8 traversal + exact fp32 rerank */
  uint32_t filter_scan_permille; /* precision 1 / 2: requests whose filter allows at most this many
                                    per mille of the nodes take the exact tensor-core scan (0: off) */
  uint32_t rerank_factor;        /* precision 1 / 2: exact rerank of the best rerank_factor x k pool
                                    entries (at least 32); 0 = the whole pool */
  uint32_t warps_per_query;      /* precision 1 / 2, dim <= 128: 4 = four warps walk each query
                                    (beam search, lower latency); 0 / 1 = one warp */
  uint32_t lists_per_step;       /* precision 1 / 2, dim <= 128: one warp per query, a beam search
                                    expanding this many lists per step (1..4); 0 = off */
  uint32_t filter_scan_mode;     /* HG_SCAN_*: the exact scan of routed requests */
} hg_server_config;
typedef struct {
  const float* queries;        /* nq x dim */
  uint32_t nq;
  uint32_t k;
  uint32_t ef;                 /* 0 = the index's set_ef value */
  uint32_t reserved;
  const hg_filter* filter;     /* NULL = none */
  hg_neighbor* out;            /* nq x k, padded like search_batch */
} hg_request;
typedef struct {
  uint64_t requests, queries, batches, memory_waits;
  double elapsed_s, qps;       /* first arrival to last completion */
  double p50_ms, p99_ms, p999_ms, mean_ms, max_ms;  /* request latency, arrival to completion */
  double mean_batch_queries;
} hg_server_stats;

int hg_server_create(const hg_index* idx, const hg_server_config* cfg, hg_server** out);
int hg_server_submit(hg_server* s, const hg_request* r, uint64_t* ticket);
int hg_server_wait(hg_server* s, uint64_t ticket, double* latency_ms);
/* Submits request i at arrival_s[i] seconds after the call (an open-loop
 * load), waits for all and reports these requests' statistics. */
int hg_server_replay(hg_server* s, const hg_request* reqs, const double* arrival_s, size_t n,
                     hg_server_stats* stats);
/* The same, also writing each request's latency (arrival to completion, ms)
 * into latency_ms[i] (n entries; NULL: none). */
int hg_server_replay_latencies(hg_server* s, const hg_request* reqs, const double* arrival_s, size_t n,
                               hg_server_stats* stats, double* latency_ms);
int hg_server_stats_get(hg_server* s, hg_server_stats* out);
void hg_server_destroy(hg_server* s);

/* Distance summation order for indexes created or loaded afterwards. */
int hg_set_distance_order(int order);
int hg_get_distance_order(void);

#ifdef __cplusplus
}
#endif
#endif /* HNSWGPU_H */
