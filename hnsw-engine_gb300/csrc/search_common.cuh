// search_common.cuh -- types shared by the search kernels and their host launcher.
#pragma once
#include <cstdint>

namespace hg {

constexpr uint32_t kNoId = 0xFFFFFFFFu;
constexpr int kCounters = 8;
constexpr uint64_t kBitmapBytesCap = 1ull << 30;   // visited bitmaps per workspace
constexpr uint64_t kPoolBytesCap = 1ull << 30;     // first-tier pools per workspace
constexpr uint64_t kBigPoolBytesCap = 2ull << 30;  // second-tier pools per workspace
constexpr uint32_t kBigPoolTries = 8192;  // bounded wait (~2 us steps) for a second-tier pool
enum : uint32_t { kTierBitmap = 1u, kTierPool = 2u, kTierRerun = 4u, kTierPool2 = 8u };

// Everything one launch of the query kernel reads.  Device pointers unless noted.
struct SearchParams {
  // ---- graph (resident) ----
  const float* vecs;        // n x pd, 64-byte rows, prepared (cosine: unit)
  const uint32_t* l0;       // n x l0_stride neighbour ids, kNoId padded
  const uint32_t* up;       // upper blocks of up_stride ids, kNoId padded
  const uint32_t* up_blk;   // n: block index of level 1 (levels 1..L contiguous)
  const uint64_t* labels;   // n
  const uint32_t* alive;    // n bits: 1 = not deleted
  uint32_t n, pd, dim, M, M0, l0_stride, up_stride;
  int32_t metric, max_level;
  uint32_t entry;
  int32_t tagged;           // n < 2^24: visited hash slots carry an 8-bit epoch
  int32_t dedup;            // some neighbour list repeats an id
  int32_t deleted_any;      // num_deleted > 0 (reference switches to the filtered variant)
  int32_t order;            // FP32 summation order: 0 the AVX-512 kernel's, 1 the NEON kernel's
  // ---- batch ----
  const float* queries;     // nq x dim raw
  uint32_t nq;
  const uint32_t* nq_dev;   // if set, nq is read from here (rerun pass)
  const uint32_t* qidx;     // if set, the i-th work item is query qidx[i]
  // one launch over all ef buckets, largest ef first: work item i maps into
  // the bucket lists qidx[b * lpt_stride ...] from bucket lpt_buckets-1 down
  const uint32_t* lpt_sizes;
  uint32_t lpt_buckets, lpt_stride;
  const uint32_t* efq;      // per query ef (0 = default) or null
  const uint32_t* kq;       // per query k or null
  uint32_t ef_all, ef_default, k_all, k_stride;
  const uint32_t* const* fbits;  // per filter: id-space bitset (n bits)
  const int32_t* fsel;           // per query filter index (-1 none) or null
  uint32_t num_filters;
  void* out;                     // 16-byte records
  uint32_t* nres;                // per query result count or null
  uint32_t* done;                // per query: set to 1 once its output row is final (system scope) or null
  // ---- per-warp shared layout ----
  uint32_t H;  // visited hash slots (power of two)
  uint32_t R;  // result capacity (>= every ef)
  uint32_t C;  // candidate head capacity (power of two, >= 64)
  // ---- global scratch ----
  // Spill pools and visited bitmaps are either one per warp slot (owner
  // arrays null: the rerun pass) or shared: a warp acquires one with a
  // bounded CAS scan of the owner array when it first needs it and releases
  // it when its query ends; if none is free the query goes to the rerun list.
  uint64_t* pool;           // candidate spill pools, pool_cap keys each
  uint64_t pool_cap;
  uint32_t* pool_owner;     // [pool_slots] 0 = free
  uint32_t pool_slots;
  uint64_t* big_pool;       // second pool tier: big_cap keys each (null: none)
  uint64_t big_cap;
  uint32_t* big_owner;      // [big_slots] 0 = free
  uint32_t big_slots;
  uint32_t* bitmaps;        // visited bitmaps, bitmap_words each
  uint64_t bitmap_words;
  uint32_t* bm_owner;       // [bm_slots] 0 = free
  uint32_t bm_slots;
  uint32_t slot_base;       // first warp slot of this launch (per-slot mode)
  int32_t rerun;            // 1: this launch is the rerun pass (counter flag only)
  // ---- compressed traversal (FP16 / FP8-E4M3 rows) ----
  const void* vq;           // n x pdc compressed rows (halves or e4m3 bytes), zero padded
  const float* vscale;      // FP8: per-row scale (row = scale x e4m3 values)
  const float* vaux;        // per row {scale (1 for FP16), scale^2 |stored row|^2}
  uint32_t lists_per_step;  // beam walk: neighbour lists expanded per step (1..4)
  uint32_t pdc;             // compressed row length (dim rounded up to 128)
  uint32_t* pool_out;       // nq x pool_stride: final traversal pool (ids, sorted by traversal distance)
  uint32_t pool_stride;
  uint32_t* pool_n;         // nq: pool size
  uint32_t rerank_factor;   // rerank the best rerank_factor x k pool entries (>= 32); 0 = all
  uint32_t* work;           // work-queue counter (zeroed before launch)
  uint32_t* ovf_list;       // queries whose pool overflowed
  uint32_t* ovf_count;
  unsigned long long* counters;  // nq x kCounters or null
  uint32_t* err;                 // set to 1 if a per-query ef / k exceeds this launch's capacity
};

// ef buckets of one batch: queries with effective ef <= hi[b] go to bucket b.
constexpr int kMaxBuckets = 12;
struct BucketSpec {
  uint32_t n;
  uint32_t hi[kMaxBuckets];
};

// The beam walk (search_beam.cuh): lists per step at most, and its per-warp
// shared layout: hash[H] | beam A, B [R each] | (filtered) results A, B
// [R each] | stage [32 E] | (filtered) eligible stage [32 E] | fresh ids
// [32 E] | fresh distances [32 E] (also the query staging area: 128 floats).
constexpr int kBeamMaxE = 4;
__host__ __device__ inline uint32_t beam_warp_bytes(uint32_t H, uint32_t R, bool filt) {
  return 4u * H + 16u * R + (filt ? 16u * R : 0u) + (filt ? 2u : 1u) * 8u * 32u * kBeamMaxE + 8u * 32u * kBeamMaxE;
}
// A query's visited-hash size in the beam walk: the smallest power of two
// >= 1024 whose 5/8 load holds twice its beam and a step's lists.  A
// function of ef alone, so a query walks the same way in any batch.
__host__ __device__ inline uint32_t beam_hash_slots(uint32_t ef) {
  const uint32_t r = (ef + 31u) / 32u * 32u;
  uint32_t H = 1024;
  while (H / 8u * 5u < 2u * (r + 128u)) H <<= 1;
  return H;
}

__host__ __device__ inline uint32_t warp_smem_bytes(uint32_t H, uint32_t R, uint32_t C) {
  // hash + results + candidates (+32 slack) + two 32-entry staging arrays +
  // the warp's rarely used state (64 bytes)
  return 4u * H + 8u * R + 8u * (C + 32u) + 2u * 8u * 32u + 64u;
}

}  // namespace hg
