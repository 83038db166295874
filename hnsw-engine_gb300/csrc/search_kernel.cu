// search_kernel.cu -- the batched HNSW query path on sm_103a.
//
// One warp answers one query at a time and pulls the next query from a
// device work queue (a persistent grid).  Per query it runs exactly the
// reference's algorithm (src/search_layer.cpp:29-171):
//
//   entry distance -> greedy descent over levels L..1 (first-best, strict <)
//   -> layer-0 beam search (Alg. 2) with candidate min-order and result
//   max-order on (distance, internal id) -> first min(k, |res|) results.
//
// Exactness.  Results are bit-identical to the reference CPU code because
//   * distances reproduce the reference kernel's summation order: the
//     AVX-512 layout (4 x 16 accumulators over 64-float blocks, 16-float
//     blocks into acc0, (acc0+acc1)+(acc2+acc3), 16->8->4->2->1 reduction;
//     src/kernels_avx512.cpp:10-58) maps onto a warp as two FMA chains per
//     lane followed by a 16/8/4/2/1 shuffle butterfly;
//   * candidates and results are totally ordered by the 64-bit key
//     (order-preserving float bits << 32 | id), so the set popped / kept is
//     independent of the data structure (index_impl.hpp:58-71);
//   * the accept test `|res| < ef || d < worst` (search_layer.cpp:120) is
//     replayed in neighbour-list order against the evolving worst result;
//   * the visited set is exact: a shared-memory open-addressing hash with an
//     8-bit epoch tag per slot, switched to a per-warp global bitmap when it
//     passes 5/8 load;
//   * candidates whose distance exceeds the current worst result once the
//     result set is full are dropped: such a candidate can only ever be
//     popped to end the loop, which an empty queue or any later candidate
//     does identically.  All other candidates are kept: a sorted head in
//     shared memory plus an unsorted spill pool in global memory
//     (invariant: every pool key > every head key).
//
// Shared memory per warp: visited hash (4H B), results (8R B), candidate head
// (8(C+32) B) and two 32-entry staging arrays.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "search_common.cuh"

namespace hg {
namespace {

constexpr unsigned kFull = 0xFFFFFFFFu;
constexpr uint64_t kMaxKey = ~0ull;

// ---------------------------------------------------------------------------
// keys: order-preserving float bits, then id
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t okey(float d) {
  d = __fadd_rn(d, 0.0f);  // -0 -> +0: key order must equal float order
  const uint32_t u = __float_as_uint(d);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float key_dist(uint64_t key) {
  const uint32_t k = static_cast<uint32_t>(key >> 32);
  const uint32_t u = (k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k;
  return __uint_as_float(u);
}
__device__ __forceinline__ uint64_t mkkey(float d, uint32_t id) {
  return (static_cast<uint64_t>(okey(d)) << 32) | id;
}
__device__ __forceinline__ uint64_t shfl64(uint64_t v, int src) {
  const uint32_t lo = __shfl_sync(kFull, static_cast<uint32_t>(v), src);
  const uint32_t hi = __shfl_sync(kFull, static_cast<uint32_t>(v >> 32), src);
  return (static_cast<uint64_t>(hi) << 32) | lo;
}
__device__ __forceinline__ uint64_t warp_max64(uint64_t v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const uint32_t lo = __shfl_xor_sync(kFull, static_cast<uint32_t>(v), o);
    const uint32_t hi = __shfl_xor_sync(kFull, static_cast<uint32_t>(v >> 32), o);
    const uint64_t w = (static_cast<uint64_t>(hi) << 32) | lo;
    v = w > v ? w : v;
  }
  return v;
}
__device__ __forceinline__ float warp_minf(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(kFull, v, o));
  return v;
}

// number of elements of sorted a[0..n) that are < x
__device__ __forceinline__ int lower_bound(const uint64_t* a, int n, uint64_t x) {
  int lo = 0, hi = n;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (a[mid] < x) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// Merge sorted b[0..m) into sorted a[0..n) in place (keys unique), keeping
// the smallest `cap`.  Returns the new size.  Whole warp, uniform arguments.
__device__ int warp_merge(uint64_t* a, int n, int cap, const uint64_t* b, int m, int lane) {
  if (m == 0) return n;
  int rb = 0;
  uint64_t bj = 0;
  if (lane < m) {
    bj = b[lane];
    rb = lower_bound(a, n, bj);
  }
  const int p0 = __shfl_sync(kFull, rb, 0);
  for (int top = n; top > p0; top -= 32) {
    const int p = top - 32 + lane;
    uint64_t x = 0;
    int dst = -1;
    if (p >= p0 && p < n) {
      x = a[p];
      dst = p + lower_bound(b, m, x);
    }
    __syncwarp();
    if (dst >= 0 && dst < cap) a[dst] = x;
    __syncwarp();
  }
  if (lane < m) {
    const int dst = lane + rb;
    if (dst < cap) a[dst] = bj;
  }
  __syncwarp();
  const int t = n + m;
  return t < cap ? t : cap;
}

// Bitonic sort of a[0..p2) (p2 a power of two) by one warp.
__device__ void warp_bitonic(uint64_t* a, int p2, int lane) {
  for (int k = 2; k <= p2; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = lane; i < p2; i += 32) {
        const int l = i ^ j;
        if (l > i) {
          const uint64_t x = a[i], y = a[l];
          const bool up = (i & k) == 0;
          if ((x > y) == up) {
            a[i] = y;
            a[l] = x;
          }
        }
      }
      __syncwarp();
    }
  }
}

// ---------------------------------------------------------------------------
// distances in the AVX-512 kernel's order.  Lane t holds query elements
//   slot i < nb:        64 i + t        (chain A: acc0 lanes t<16 / acc1 t>=16)
//   slot nb + i < 2nb:  64 i + 32 + t   (chain B: acc2 / acc3)
//   slot 2nb + u < 2nb+nt, t < 16: 64 nb + 16 u + t  (16-float blocks -> acc0)
// ---------------------------------------------------------------------------
__device__ __forceinline__ int slot_elem(int i, int nb, int nt, int lane) {
  if (i < nb) return 64 * i + lane;
  if (i < 2 * nb) return 64 * (i - nb) + 32 + lane;
  const int u = i - 2 * nb;
  if (u < nt && lane < 16) return 64 * nb + 16 * u + lane;
  return -1;
}

template <int S, bool L2>
__device__ __forceinline__ float combine(const float (&x)[S], const float (&qr)[S], int nb, int nt) {
  float a = 0.0f, b = 0.0f;
#pragma unroll
  for (int i = 0; i < S; ++i) {
    if (i < nb) {
      if (L2) {
        const float d = __fsub_rn(qr[i], x[i]);
        a = __fmaf_rn(d, d, a);
      } else {
        a = __fmaf_rn(qr[i], x[i], a);
      }
    }
  }
#pragma unroll
  for (int i = 0; i < S; ++i) {
    if (i >= nb && i < 2 * nb) {
      if (L2) {
        const float d = __fsub_rn(qr[i], x[i]);
        b = __fmaf_rn(d, d, b);
      } else {
        b = __fmaf_rn(qr[i], x[i], b);
      }
    }
  }
#pragma unroll
  for (int i = 0; i < S; ++i) {
    if (i >= 2 * nb && i < 2 * nb + nt) {  // lanes >= 16 hold zeros here
      if (L2) {
        const float d = __fsub_rn(qr[i], x[i]);
        a = __fmaf_rn(d, d, a);
      } else {
        a = __fmaf_rn(qr[i], x[i], a);
      }
    }
  }
  // (acc0 + acc1) + (acc2 + acc3), then the 16-lane reduction
  const float xa = __fadd_rn(a, __shfl_xor_sync(kFull, a, 16));
  const float xb = __fadd_rn(b, __shfl_xor_sync(kFull, b, 16));
  float s = __fadd_rn(xa, xb);
  s = __fadd_rn(s, __shfl_xor_sync(kFull, s, 8));
  s = __fadd_rn(s, __shfl_xor_sync(kFull, s, 4));
  s = __fadd_rn(s, __shfl_xor_sync(kFull, s, 2));
  s = __fadd_rn(s, __shfl_xor_sync(kFull, s, 1));
  return L2 ? s : __fsub_rn(1.0f, s);
}

// Distances from the query to up to G rows (ids; kNoId = unused), all lanes
// get every result.  All loads are issued before any arithmetic.
template <int S, int G, bool L2>
__device__ __forceinline__ void group_dist(const float* __restrict__ vecs, uint32_t pd, const uint32_t (&ids)[G],
                                           const float (&qr)[S], int nb, int nt, int lane, float (&out)[G]) {
  float x[G][S];
#pragma unroll
  for (int g = 0; g < G; ++g) {
    const float* row = vecs + static_cast<size_t>(ids[g] == kNoId ? 0u : ids[g]) * pd;
#pragma unroll
    for (int i = 0; i < S; ++i) {
      const int e = slot_elem(i, nb, nt, lane);
      x[g][i] = (ids[g] != kNoId && e >= 0) ? __ldg(row + e) : 0.0f;
    }
  }
#pragma unroll
  for (int g = 0; g < G; ++g) out[g] = combine<S, L2>(x[g], qr, nb, nt);
}

// Distances for the lanes in `mask`; lane j receives the distance of its id.
template <int S, int G, bool L2>
__device__ __forceinline__ float lane_dists(const float* __restrict__ vecs, uint32_t pd, uint32_t id, uint32_t mask,
                                            const float (&qr)[S], int nb, int nt, int lane) {
  float mine = 0.0f;
  while (mask) {
    uint32_t gid[G];
    int gl[G];
#pragma unroll
    for (int g = 0; g < G; ++g) {
      if (mask) {
        const int l = __ffs(mask) - 1;
        mask &= mask - 1;
        gl[g] = l;
      } else {
        gl[g] = -1;
      }
      gid[g] = __shfl_sync(kFull, id, gl[g] < 0 ? 0 : gl[g]);
      if (gl[g] < 0) gid[g] = kNoId;
    }
    float gd[G];
    group_dist<S, G, L2>(vecs, pd, gid, qr, nb, nt, lane, gd);
#pragma unroll
    for (int g = 0; g < G; ++g)
      if (gl[g] == lane) mine = gd[g];
  }
  return mine;
}

// ---------------------------------------------------------------------------
// per-warp state
// ---------------------------------------------------------------------------
struct Warp {
  uint32_t* hash;
  uint64_t* res;
  uint64_t* cand;
  uint64_t* stA;
  uint64_t* stE;
  uint64_t* pool;     // this slot's spill pool
  uint32_t* bitmap;   // this slot's visited bitmap
  uint32_t hmask;
  int hshift;
  uint32_t tag;       // epoch << 24 (tagged mode)
  uint32_t vcount;    // visited entries in the hash
  bool bitmap_mode;
};

__device__ __forceinline__ bool hash_empty(uint32_t v, uint32_t tag, bool tagged) {
  return tagged ? ((v & 0xFF000000u) != tag) : (v == kNoId);
}

// Test-and-mark `id` (valid lanes only); returns true if it was visited.
__device__ __forceinline__ bool visit(Warp& w, uint32_t id, bool tagged) {
  if (w.bitmap_mode) {
    const uint32_t bit = 1u << (id & 31u);
    const uint32_t old = atomicOr(&w.bitmap[id >> 5], bit);
    return (old & bit) != 0;
  }
  const uint32_t key = tagged ? (w.tag | id) : id;
  uint32_t p = (id * 0x9E3779B1u) >> w.hshift;
  for (;;) {
    const uint32_t v = *reinterpret_cast<volatile const uint32_t*>(&w.hash[p]);
    if (!hash_empty(v, w.tag, tagged)) {
      if (v == key) return true;
      p = (p + 1) & w.hmask;
      continue;
    }
    const uint32_t old = atomicCAS(&w.hash[p], v, key);
    if (old == v) return false;
    if (old == key) return true;
  }
}

// Move the visited set from the hash to this slot's bitmap.
__device__ void to_bitmap(Warp& w, const SearchParams& P, bool tagged, int lane) {
  const uint64_t words = P.bitmap_words;
  for (uint64_t i = lane; i < words; i += 32) w.bitmap[i] = 0u;
  __syncwarp();
  __threadfence_block();
  for (uint32_t p = lane; p <= w.hmask; p += 32) {
    const uint32_t v = w.hash[p];
    if (!hash_empty(v, w.tag, tagged)) {
      const uint32_t id = tagged ? (v & 0x00FFFFFFu) : v;
      atomicOr(&w.bitmap[id >> 5], 1u << (id & 31u));
    }
  }
  __threadfence_block();
  __syncwarp();
  w.bitmap_mode = true;
}

__device__ __forceinline__ bool bit_of(const uint32_t* bits, uint32_t id) {
  return ((__ldg(bits + (id >> 5)) >> (id & 31u)) & 1u) != 0;
}

// Radix select: the r-th smallest (1-based) of pool[0..pn).  hist: 256 u32 in smem.
__device__ uint64_t radix_select(const uint64_t* pool, uint64_t pn, uint64_t r, uint32_t* hist, int lane) {
  uint64_t prefix = 0, pmask = 0;
  for (int shift = 56; shift >= 0; shift -= 8) {
    for (int i = lane; i < 256; i += 32) hist[i] = 0u;
    __syncwarp();
    for (uint64_t i = lane; i < pn; i += 32) {
      const uint64_t x = pool[i];
      if ((x & pmask) == prefix) atomicAdd(&hist[(x >> shift) & 255u], 1u);
    }
    __syncwarp();
    // lane l owns bins 8l..8l+7
    uint32_t c[8];
    uint32_t tot = 0;
#pragma unroll
    for (int b = 0; b < 8; ++b) {
      c[b] = hist[8 * lane + b];
      tot += c[b];
    }
    uint32_t incl = tot;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t v = __shfl_up_sync(kFull, incl, o);
      if (lane >= o) incl += v;
    }
    const uint32_t excl = incl - tot;
    const bool here = excl < r && r <= incl;
    const uint32_t owner_mask = __ballot_sync(kFull, here);
    const int owner = __ffs(owner_mask) - 1;
    uint32_t bucket = 0, before = 0;
    if (lane == owner) {
      uint32_t cum = excl;
#pragma unroll
      for (int b = 0; b < 8; ++b) {
        if (cum + c[b] >= r) {
          bucket = 8 * lane + b;
          before = cum;
          break;
        }
        cum += c[b];
      }
    }
    bucket = __shfl_sync(kFull, bucket, owner);
    before = __shfl_sync(kFull, before, owner);
    prefix |= static_cast<uint64_t>(bucket) << shift;
    pmask |= 0xFFull << shift;
    r -= before;
    __syncwarp();
  }
  return prefix;
}

// Candidate queue: head = sorted cand[ch, ct) in smem, pool = unsorted spill.
struct Cands {
  int ch, ct;
  uint64_t pn;       // pool entries
  uint64_t pmin;     // min key in pool (kMaxKey if empty)
  uint64_t peak;     // largest head + pool size seen
  bool overflow;
};

__device__ __forceinline__ bool pool_append(Warp& w, Cands& c, const uint64_t* src, int cnt, uint64_t cap, int lane) {
  if (cnt <= 0) return true;
  if (c.pn + static_cast<uint64_t>(cnt) > cap) {
    c.overflow = true;
    return false;
  }
  if (lane < cnt) w.pool[c.pn + lane] = src[lane];
  c.pn += cnt;
  return true;
}

// Refill an empty head from the pool with its smallest C/2 keys; when the
// result set is full, first drop pool keys farther than the worst result.
__device__ void refill(Warp& w, Cands& c, const SearchParams& P, bool res_full, float worst_d, int lane) {
  __threadfence_block();
  if (res_full) {
    uint64_t wpos = 0;
    for (uint64_t base = 0; base < c.pn; base += 32) {
      const uint64_t i = base + lane;
      uint64_t x = 0;
      bool keep = false;
      if (i < c.pn) {
        x = w.pool[i];
        keep = key_dist(x) <= worst_d;
      }
      const uint32_t bal = __ballot_sync(kFull, keep);
      __syncwarp();
      if (keep) w.pool[wpos + __popc(bal & ((1u << lane) - 1u))] = x;
      wpos += __popc(bal);
      __syncwarp();
    }
    c.pn = wpos;
  }
  c.ch = c.ct = 0;
  c.pmin = kMaxKey;
  if (c.pn == 0) return;
  const uint64_t half = P.C / 2;
  const uint64_t take = c.pn < half ? c.pn : half;
  uint64_t T = kMaxKey;
  if (c.pn > take) T = radix_select(w.pool, c.pn, take, reinterpret_cast<uint32_t*>(w.cand), lane);
  __syncwarp();
  // split: keys <= T to the head, the rest stay (compacted) in the pool
  uint64_t hpos = 0, wpos = 0, newmin = kMaxKey;
  for (uint64_t base = 0; base < c.pn; base += 32) {
    const uint64_t i = base + lane;
    uint64_t x = kMaxKey;
    const bool live = i < c.pn;
    if (live) x = w.pool[i];
    const bool sel = live && x <= T;
    const bool rest = live && !sel;
    const uint32_t bs = __ballot_sync(kFull, sel);
    const uint32_t br = __ballot_sync(kFull, rest);
    __syncwarp();
    const uint32_t below = (1u << lane) - 1u;
    if (sel) w.cand[hpos + __popc(bs & below)] = x;
    if (rest) {
      w.pool[wpos + __popc(br & below)] = x;
      newmin = x < newmin ? x : newmin;
    }
    hpos += __popc(bs);
    wpos += __popc(br);
    __syncwarp();
  }
  newmin = ~warp_max64(~newmin);
  int p2 = 1;
  while (p2 < static_cast<int>(hpos)) p2 <<= 1;
  for (int i = static_cast<int>(hpos) + lane; i < p2; i += 32) w.cand[i] = kMaxKey;
  __syncwarp();
  warp_bitonic(w.cand, p2, lane);
  c.ct = static_cast<int>(hpos);
  c.pn = wpos;
  c.pmin = wpos ? newmin : kMaxKey;
  __threadfence_block();
}

// Insert the sorted accepted batch stA[0..m) into the candidate queue.
// res_full / worst_d: once the result set is full, head keys farther than the
// worst result are dropped before anything would spill to the pool.
__device__ void cand_insert(Warp& w, Cands& c, const SearchParams& P, int m, bool res_full, float worst_d,
                            int lane) {
  if (m <= 0) return;
  if (res_full && c.ct - c.ch + m > static_cast<int>(P.C) - c.ch) {
    // first head index whose distance exceeds the worst result
    int lo = c.ch, hi = c.ct;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (key_dist(w.cand[mid]) > worst_d) hi = mid;
      else lo = mid + 1;
    }
    c.ct = lo;
  }
  int mh = m;
  if (c.pn > 0) {
    const bool lt = lane < m && w.stA[lane] < c.pmin;
    mh = __popc(__ballot_sync(kFull, lt));
    if (m > mh && !pool_append(w, c, w.stA + mh, m - mh, P.pool_cap, lane)) return;
  }
  if (mh > 0) {
    const int n = c.ct - c.ch;
    const int nn = warp_merge(w.cand + c.ch, n, static_cast<int>(P.C) + 32 - c.ch, w.stA, mh, lane);
    c.ct = c.ch + nn;
    if (c.ct > static_cast<int>(P.C)) {
      if (c.ch > 0) {  // compact to the front
        const int len = c.ct - c.ch;
        for (int base = 0; base < len; base += 32) {
          const int i = base + lane;
          uint64_t x = 0;
          if (i < len) x = w.cand[c.ch + i];
          __syncwarp();
          if (i < len) w.cand[i] = x;
          __syncwarp();
        }
        c.ct = len;
        c.ch = 0;
      }
      if (c.ct > static_cast<int>(P.C)) {  // spill the largest keys
        const int cnt = c.ct - static_cast<int>(P.C);
        const uint64_t first = w.cand[P.C];
        if (!pool_append(w, c, w.cand + P.C, cnt, P.pool_cap, lane)) return;
        c.pmin = first < c.pmin ? first : c.pmin;
        c.ct = static_cast<int>(P.C);
      }
    }
  }
  const uint64_t total = static_cast<uint64_t>(c.ct - c.ch) + c.pn;
  c.peak = total > c.peak ? total : c.peak;
}

struct QueryOut {
  uint64_t label;
  float dist;
  uint32_t zero;
};

// ---------------------------------------------------------------------------
// the kernel
// ---------------------------------------------------------------------------
template <int S, int G, bool L2>
__global__ void __launch_bounds__(128) search_kernel(SearchParams P, const float* __restrict__ inv_norm) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const uint32_t per_warp = warp_smem_bytes(P.H, P.R, P.C);
  unsigned char* base = smem + static_cast<size_t>(wib) * per_warp;
  const uint64_t slot = static_cast<uint64_t>(blockIdx.x) * (blockDim.x >> 5) + wib;

  Warp w;
  w.hash = reinterpret_cast<uint32_t*>(base);
  w.res = reinterpret_cast<uint64_t*>(base + 4u * P.H);
  w.cand = w.res + P.R;
  w.stA = w.cand + P.C + 32;
  w.stE = w.stA + 32;
  w.pool = P.pool + slot * P.pool_cap;
  w.bitmap = P.bitmaps + slot * P.bitmap_words;
  w.hmask = P.H - 1;
  w.hshift = 32 - (31 - __clz(P.H));
  const bool tagged = P.tagged != 0;
  uint32_t epoch = 0;
  for (uint32_t i = lane; i < P.H; i += 32) w.hash[i] = tagged ? 0u : kNoId;
  __syncwarp();

  const int nb = static_cast<int>(P.pd / 64);
  const int nt = static_cast<int>((P.pd % 64) / 16);
  const uint32_t nq = P.nq_dev ? *P.nq_dev : P.nq;

  for (;;) {
    uint32_t item = 0;
    if (lane == 0) item = atomicAdd(P.work, 1u);
    item = __shfl_sync(kFull, item, 0);
    if (item >= nq) break;
    const uint32_t q = P.qidx ? P.qidx[item] : item;

    uint32_t k = P.kq ? P.kq[q] : P.k_all;
    uint32_t ef = P.efq ? P.efq[q] : P.ef_all;
    if (ef == 0) ef = P.ef_default;
    if (ef < k) ef = k;
    if (ef > P.R || k > P.k_stride || k == 0) {
      // device-side arrays promised a smaller bound: refuse this query
      if (lane == 0) atomicExch(P.err, 1u);
      continue;
    }
    const uint32_t* fb = nullptr;
    if (P.fsel) {
      const int32_t f = P.fsel[q];
      if (f >= 0) fb = P.fbits[f];
    }
    const bool filtered = fb != nullptr || P.deleted_any != 0;
    unsigned long long cnt[kCounters] = {0, 0, 0, 0, 0, 0, 0, 0};

    int s = 0;  // result count
    Cands c{0, 0, 0, kMaxKey, 0, false};
    if (P.n > 0) {
      // ---- query registers (prepare_vector: cosine scaled by 1/||q||) ----
      const float* raw = P.queries + static_cast<size_t>(q) * P.dim;
      const float inv = inv_norm ? inv_norm[q] : 1.0f;
      float qr[S];
#pragma unroll
      for (int i = 0; i < S; ++i) {
        const int e = slot_elem(i, nb, nt, lane);
        const float v = (e >= 0 && e < static_cast<int>(P.dim)) ? __ldg(raw + e) : 0.0f;
        qr[i] = inv_norm ? __fmul_rn(v, inv) : v;
      }
      // ---- visited set for this query ----
      w.bitmap_mode = false;
      w.vcount = 0;
      if (tagged) {
        if (++epoch == 256u) {
          for (uint32_t i = lane; i < P.H; i += 32) w.hash[i] = 0u;
          __syncwarp();
          epoch = 1;
        }
        w.tag = epoch << 24;
      } else {
        for (uint32_t i = lane; i < P.H; i += 32) w.hash[i] = kNoId;
        __syncwarp();
        w.tag = 0;
      }

      // ---- entry point + greedy descent (search_layer.cpp:29-56,156-157) ----
      uint32_t cur = P.entry;
      float cur_d = lane_dists<S, G, L2>(P.vecs, P.pd, cur, 1u, qr, nb, nt, lane);
      cur_d = __shfl_sync(kFull, cur_d, 0);
      cnt[1]++;
      for (int lc = P.max_level; lc > 0; --lc) {
        bool changed = true;
        while (changed) {
          changed = false;
          const uint32_t* lst = P.up + static_cast<size_t>(P.up_blk[cur] + (lc - 1)) * P.up_stride;
          cnt[0]++;
          for (uint32_t c0 = 0; c0 < P.M; c0 += 32) {
            const uint32_t j = c0 + lane;
            const uint32_t id = j < P.M ? __ldg(lst + j) : kNoId;
            const uint32_t vm = __ballot_sync(kFull, id != kNoId);
            if (!vm) break;
            cnt[1] += __popc(vm);
            const float d = lane_dists<S, G, L2>(P.vecs, P.pd, id, vm, qr, nb, nt, lane);
            const float m = warp_minf(id != kNoId ? d : __int_as_float(0x7f800000));
            if (m < cur_d) {
              const uint32_t hit = __ballot_sync(kFull, id != kNoId && d == m);
              const int l = __ffs(hit) - 1;
              cur = __shfl_sync(kFull, id, l);
              cur_d = m;
              changed = true;
            }
          }
        }
      }

      // ---- layer 0 (search_layer.cpp:58-134) ----
      if (lane == 0) visit(w, cur, tagged);
      __syncwarp();
      w.vcount = 1;
      cnt[4] = 1;
      const uint64_t k0 = mkkey(cur_d, cur);
      if (lane == 0) {
        w.cand[0] = k0;
        if (!filtered || (bit_of(P.alive, cur) && (!fb || bit_of(fb, cur)))) w.res[0] = k0;
      }
      c.ct = 1;
      c.peak = 1;
      if (!filtered || (bit_of(P.alive, cur) && (!fb || bit_of(fb, cur)))) s = 1;
      __syncwarp();

      const uint32_t hlimit = (P.H * 5u) / 8u;
      for (;;) {
        if (c.ch == c.ct) {
          if (c.pn == 0) break;
          const bool full = s >= static_cast<int>(ef);
          refill(w, c, P, full, full ? key_dist(w.res[s - 1]) : 0.0f, lane);
          if (c.ch == c.ct) break;
        }
        const uint64_t top = w.cand[c.ch];
        if (s >= static_cast<int>(ef) && key_dist(top) > key_dist(w.res[s - 1])) break;
        c.ch++;
        const uint32_t cid = static_cast<uint32_t>(top);
        const uint32_t* lst = P.l0 + static_cast<size_t>(cid) * P.l0_stride;
        cnt[2]++;
        for (uint32_t c0 = 0; c0 < P.M0; c0 += 32) {
          const uint32_t j = c0 + lane;
          const uint32_t id = j < P.M0 ? __ldg(lst + j) : kNoId;
          const bool valid = id != kNoId;
          const uint32_t vm = __ballot_sync(kFull, valid);
          if (!vm) break;
          if (!w.bitmap_mode && w.vcount + __popc(vm) > hlimit) to_bitmap(w, P, tagged, lane);
          bool first = valid;
          if (P.dedup && valid) {
            const uint32_t same = __match_any_sync(vm, id);
            first = (__ffs(same) - 1) == lane;
          }
          bool fresh = false;
          if (first) fresh = !visit(w, id, tagged);
          __syncwarp();
          uint32_t U = __ballot_sync(kFull, fresh);
          w.vcount += __popc(U);
          cnt[4] += __popc(U);
          if (!U) continue;
          cnt[3] += __popc(U);
          const float d = lane_dists<S, G, L2>(P.vecs, P.pd, id, U, qr, nb, nt, lane);
          bool elig = true;
          if (filtered && fresh) elig = bit_of(P.alive, id) && (!fb || bit_of(fb, id));
          const uint64_t key = mkkey(d, id);

          // ---- in-order acceptance replay ----
          const int s0 = s;
          uint32_t acc = 0, ins = 0, inres = 0;
          int scur = s0, r = s0 - 1;
          float worst_d = 0.0f;
          if (s0 >= static_cast<int>(ef)) {
            worst_d = key_dist(w.res[s0 - 1]);
            U &= __ballot_sync(kFull, d < worst_d);
          }
          while (U) {
            const int jl = __ffs(U) - 1;
            U &= U - 1;
            const float dj = __shfl_sync(kFull, d, jl);
            const bool ej = __shfl_sync(kFull, elig, jl);
            const bool a = scur < static_cast<int>(ef) || dj < worst_d;
            if (!a) continue;
            acc |= 1u << jl;
            if (!ej) continue;
            ins |= 1u << jl;
            inres |= 1u << jl;
            if (scur < static_cast<int>(ef)) {
              ++scur;
              if (scur == static_cast<int>(ef)) {
                const uint64_t mi = warp_max64((inres >> lane) & 1u ? key : 0ull);
                const uint64_t rr = r >= 0 ? w.res[r] : 0ull;
                worst_d = key_dist(rr > mi ? rr : mi);
              }
            } else {
              uint64_t mi = warp_max64((inres >> lane) & 1u ? key : 0ull);
              const uint64_t rr = r >= 0 ? w.res[r] : 0ull;
              if (rr > mi) {
                --r;
              } else {
                const uint32_t who = __ballot_sync(kFull, ((inres >> lane) & 1u) && key == mi);
                inres &= ~who;
              }
              mi = warp_max64((inres >> lane) & 1u ? key : 0ull);
              const uint64_t r2 = r >= 0 ? w.res[r] : 0ull;
              worst_d = key_dist(r2 > mi ? r2 : mi);
            }
          }
          if (!acc) continue;

          // ---- sorted batches: all accepted (cand), eligible accepted (res) ----
          {
            int rA = 0, rE = 0;
            uint32_t it = acc;
            while (it) {
              const int i = __ffs(it) - 1;
              it &= it - 1;
              const uint64_t ki = shfl64(key, i);
              const bool lt = ki < key;
              rA += lt;
              rE += lt && ((ins >> i) & 1u);
            }
            if ((acc >> lane) & 1u) w.stA[rA] = key;
            if ((ins >> lane) & 1u) w.stE[rE] = key;
            __syncwarp();
          }
          const int mA = __popc(acc), mE = __popc(ins);
          s = warp_merge(w.res, s, static_cast<int>(ef), w.stE, mE, lane);
          int mAk = mA;
          const bool full = s >= static_cast<int>(ef);
          const float wd = full ? key_dist(w.res[s - 1]) : 0.0f;
          if (full) mAk = __popc(__ballot_sync(kFull, lane < mA && key_dist(w.stA[lane]) <= wd));
          cand_insert(w, c, P, mAk, full, wd, lane);
          if (c.overflow) break;
        }
        if (c.overflow) break;
      }
    }

    if (c.overflow) {
      if (lane == 0) {
        const uint32_t o = atomicAdd(P.ovf_count, 1u);
        P.ovf_list[o] = q;
      }
      continue;
    }

    // ---- output (search_layer.cpp:166-169, 189-192) ----
    const int m = s < static_cast<int>(k) ? s : static_cast<int>(k);
    QueryOut* row = static_cast<QueryOut*>(P.out) + static_cast<size_t>(q) * P.k_stride;
    for (uint32_t j = lane; j < P.k_stride; j += 32) {
      QueryOut o;
      if (static_cast<int>(j) < m) {
        const uint64_t kk = w.res[j];
        o.label = P.labels[static_cast<uint32_t>(kk)];
        o.dist = key_dist(kk);
      } else {
        o.label = ~0ull;
        o.dist = __int_as_float(0x7f800000);
      }
      o.zero = 0;
      row[j] = o;
    }
    if (P.nres && lane == 0) P.nres[q] = static_cast<uint32_t>(m);
    if (P.counters && lane == 0) {
      cnt[5] = c.peak;
      cnt[6] = static_cast<unsigned long long>(s);
      cnt[7] = (w.bitmap_mode ? kTierBitmap : 0u) | (c.peak > P.C ? kTierPool : 0u) | (P.qidx ? kTierRerun : 0u);
      for (int i = 0; i < kCounters; ++i) P.counters[static_cast<size_t>(q) * kCounters + i] = cnt[i];
    }
    __syncwarp();
  }
}

// Cosine: inv_norm[q] = float(1 / sqrt(sum in double, in order)) (space.hpp:31-40).
__global__ void inv_norm_kernel(const float* __restrict__ qs, uint32_t nq, uint32_t dim, float* __restrict__ out) {
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq) return;
  const float* x = qs + static_cast<size_t>(q) * dim;
  double norm = 0.0;
  for (uint32_t i = 0; i < dim; ++i) {
    const double v = static_cast<double>(x[i]);
    norm = __dadd_rn(norm, __dmul_rn(v, v));
  }
  out[q] = norm > 0.0 ? __double2float_rn(1.0 / sqrt(norm)) : 1.0f;
}

template <int S, int G>
cudaError_t launch_s(const SearchParams& P, const float* inv, int blocks, int threads, size_t smem, cudaStream_t st) {
  if (P.metric == 0) {
    auto* fn = search_kernel<S, G, true>;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    fn<<<blocks, threads, smem, st>>>(P, inv);
  } else {
    auto* fn = search_kernel<S, G, false>;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess) return e;
    fn<<<blocks, threads, smem, st>>>(P, inv);
  }
  return cudaGetLastError();
}

// Label-space BitsetFilter words -> id-space bits: bit id set iff
// labels[id] < num_bits and that label's bit is set (filter.hpp:39-41).
__global__ void translate_filter_kernel(const uint64_t* __restrict__ words, uint64_t num_bits,
                                        const uint64_t* __restrict__ labels, uint32_t n, uint32_t* __restrict__ out,
                                        uint32_t out_words) {
  const uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= out_words) return;
  uint32_t bits = 0;
  for (uint32_t b = 0; b < 32; ++b) {
    const uint64_t id = static_cast<uint64_t>(w) * 32 + b;
    if (id >= n) break;
    const uint64_t l = labels[id];
    if (l < num_bits && ((words[l >> 6] >> (l & 63)) & 1ull)) bits |= 1u << b;
  }
  out[w] = bits;
}

template <int S, int G>
int occupancy_s(int metric, int threads, size_t smem) {
  int blocks = 0;
  if (metric == 0) {
    auto* fn = search_kernel<S, G, true>;
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)) != cudaSuccess)
      return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, fn, threads, smem) != cudaSuccess) return 0;
  } else {
    auto* fn = search_kernel<S, G, false>;
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)) != cudaSuccess)
      return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, fn, threads, smem) != cudaSuccess) return 0;
  }
  return blocks;
}

}  // namespace

// Query slots per lane for padded dim pd (AVX-512 layout).
int slots_for(uint32_t pd) { return 2 * static_cast<int>(pd / 64) + static_cast<int>((pd % 64) / 16); }

cudaError_t launch_inv_norm(const float* qs, uint32_t nq, uint32_t dim, float* out, cudaStream_t st) {
  if (nq == 0) return cudaSuccess;
  inv_norm_kernel<<<(nq + 127) / 128, 128, 0, st>>>(qs, nq, dim, out);
  return cudaGetLastError();
}

// Returns cudaErrorInvalidValue for a padded dimension beyond the register layouts.
cudaError_t launch_search(const SearchParams& P, const float* inv, int blocks, int warps_per_block,
                          cudaStream_t st) {
  const size_t smem = static_cast<size_t>(warps_per_block) * warp_smem_bytes(P.H, P.R, P.C);
  const int threads = 32 * warps_per_block;
  const int S = slots_for(P.pd);
  if (S <= 5) return launch_s<5, 8>(P, inv, blocks, threads, smem, st);
  if (S <= 9) return launch_s<9, 4>(P, inv, blocks, threads, smem, st);
  if (S <= 17) return launch_s<17, 2>(P, inv, blocks, threads, smem, st);
  if (S <= 33) return launch_s<33, 1>(P, inv, blocks, threads, smem, st);
  return cudaErrorInvalidValue;
}

}  // namespace hg

namespace hg {

cudaError_t launch_translate_filter(const uint64_t* label_words, uint64_t num_bits, const uint64_t* labels, uint32_t n,
                                    uint32_t* out, cudaStream_t st) {
  const uint32_t out_words = (n + 31) / 32 + 1;
  translate_filter_kernel<<<(out_words + 255) / 256, 256, 0, st>>>(label_words, num_bits, labels, n, out, out_words);
  return cudaGetLastError();
}

// Resident blocks per SM of the search kernel for this shape (0 on error).
int search_occupancy(uint32_t pd, int metric, int warps_per_block, uint32_t H, uint32_t R, uint32_t C) {
  const size_t smem = static_cast<size_t>(warps_per_block) * warp_smem_bytes(H, R, C);
  const int threads = 32 * warps_per_block;
  const int S = slots_for(pd);
  if (S <= 5) return occupancy_s<5, 8>(metric, threads, smem);
  if (S <= 9) return occupancy_s<9, 4>(metric, threads, smem);
  if (S <= 17) return occupancy_s<17, 2>(metric, threads, smem);
  if (S <= 33) return occupancy_s<33, 1>(metric, threads, smem);
  return 0;
}

}  // namespace hg

// ---------------------------------------------------------------------------
// Batches that allocate nothing.
//
// Some callers cannot call cudaMalloc while they search: a serving process
// that hands the GPU to other work under a fixed memory budget, code running
// inside a region where allocation would synchronise the device or is
// forbidden, or a host framework that owns every device allocation itself.
// For them the search kernel also runs with its scratch (work counters, spill
// pools, visited bitmaps, the rerun list and the cosine norms) placed in the
// file-scope array below instead of buffers the library allocates.  Every
// GPU that loads the library holds this array (about 15.4 MiB) until the
// process exits.
// ---------------------------------------------------------------------------
namespace hg {
namespace {

constexpr uint32_t kNaMaxNodes = 1u << 20;    // largest graph
constexpr uint32_t kNaMaxQueries = 1u << 16;  // largest batch
constexpr uint32_t kNaMaxEf = 512;            // largest ef (after max(ef, k))
constexpr int kNaWarpsPerBlock = 4;
constexpr int kNaBlocks = 12;
constexpr uint64_t kNaSlots = static_cast<uint64_t>(kNaWarpsPerBlock) * kNaBlocks;
constexpr uint64_t kNaPoolCap = 2048;                    // spill keys per warp before the rerun pass
constexpr uint64_t kNaBitmapWords = kNaMaxNodes / 32 + 1;

// byte layout of the array
constexpr size_t kNaOffCounters = 0;  // u32: [0] work, [1] overflow count, [2] rerun work, [3] spare, [4] error
constexpr size_t kNaOffOvf = 256;
constexpr size_t kNaOffInv = kNaOffOvf + 4ull * kNaMaxQueries;
constexpr size_t kNaOffPool = kNaOffInv + 4ull * kNaMaxQueries;
constexpr size_t kNaOffBitmaps = kNaOffPool + 8ull * kNaSlots * kNaPoolCap;
constexpr size_t kNaOffBigPool = kNaOffBitmaps + 4ull * kNaSlots * kNaBitmapWords;
constexpr size_t kNaOffBigBitmap = kNaOffBigPool + 8ull * kNaMaxNodes;
constexpr size_t kNaBytes = kNaOffBigBitmap + 4ull * kNaBitmapWords;
static_assert(kNaOffPool % 8 == 0 && kNaOffBigPool % 8 == 0, "8-byte keys need 8-byte alignment");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNaBytes];

std::mutex g_na_mutex;
void* g_na_address[64] = {};

// Device address of the array on the current device, looked up once per
// device (host code cannot use the symbol itself as a device pointer).
cudaError_t noalloc_scratch(int device, unsigned char** out) {
  if (device < 0 || device >= 64) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_na_mutex);
  if (g_na_address[device] == nullptr) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_na_address[device] = p;
  }
  *out = static_cast<unsigned char*>(g_na_address[device]);
  return cudaSuccess;
}

}  // namespace

uint32_t noalloc_max_nodes() { return kNaMaxNodes; }
uint32_t noalloc_max_queries() { return kNaMaxQueries; }
uint32_t noalloc_max_ef() { return kNaMaxEf; }

// Enqueue one batch with scratch from the static array.  P carries the graph
// and the batch (shape H/R/C included); its scratch fields are filled here.
// The caller made `device` current.
cudaError_t launch_search_noalloc(SearchParams P, int device, bool cosine, cudaStream_t st) {
  unsigned char* base = nullptr;
  cudaError_t e = noalloc_scratch(device, &base);
  if (e != cudaSuccess) return e;
  uint32_t* ctr = reinterpret_cast<uint32_t*>(base + kNaOffCounters);
  e = cudaMemsetAsync(ctr, 0, 256, st);  // counters and flags must start at zero
  if (e != cudaSuccess) return e;
  float* inv = nullptr;
  if (cosine) {
    inv = reinterpret_cast<float*>(base + kNaOffInv);
    e = launch_inv_norm(P.queries, P.nq, P.dim, inv, st);
    if (e != cudaSuccess) return e;
  }
  P.pool = reinterpret_cast<uint64_t*>(base + kNaOffPool);
  P.pool_cap = kNaPoolCap;
  P.bitmaps = reinterpret_cast<uint32_t*>(base + kNaOffBitmaps);
  P.bitmap_words = kNaBitmapWords;
  P.work = ctr;
  P.ovf_count = ctr + 1;
  P.ovf_list = reinterpret_cast<uint32_t*>(base + kNaOffOvf);
  P.err = ctr + 4;
  P.nq_dev = nullptr;
  P.qidx = nullptr;
  e = launch_search(P, inv, kNaBlocks, kNaWarpsPerBlock, st);
  if (e != cudaSuccess) return e;
  // queries whose spill pool overflowed: one warp with a pool of n keys
  SearchParams B = P;
  B.nq_dev = ctr + 1;
  B.qidx = P.ovf_list;
  B.work = ctr + 2;
  B.pool = reinterpret_cast<uint64_t*>(base + kNaOffBigPool);
  B.pool_cap = kNaMaxNodes;
  B.bitmaps = reinterpret_cast<uint32_t*>(base + kNaOffBigBitmap);
  B.ovf_count = ctr + 3;
  return launch_search(B, inv, 1, 1, st);
}

}  // namespace hg
