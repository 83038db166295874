// search_kernel.cuh -- the batched HNSW query kernel (templates; instantiated
// per metric in search_l2.cu / search_dot.cu).
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
#pragma once

#include <cuda_fp16.h>
#include <cuda_fp8.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "compressed_layout.cuh"
#include "search_common.cuh"
#include "smem_limit.cuh"

namespace hg {
namespace sk {

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

// Sort one 64-bit key per lane ascending across the warp (bitonic network).
__device__ __forceinline__ uint64_t warp_sort32(uint64_t v, int lane) {
#pragma unroll
  for (int k = 2; k <= 32; k <<= 1) {
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1) {
      const uint32_t lo = __shfl_xor_sync(kFull, static_cast<uint32_t>(v), j);
      const uint32_t hi = __shfl_xor_sync(kFull, static_cast<uint32_t>(v >> 32), j);
      const uint64_t o = (static_cast<uint64_t>(hi) << 32) | lo;
      const bool keep_min = ((lane & j) == 0) == ((lane & k) == 0);
      v = keep_min ? (o < v ? o : v) : (o > v ? o : v);
    }
  }
  return v;
}
__device__ __forceinline__ uint64_t warp_min64(uint64_t v) { return ~warp_max64(~v); }

// number of elements of sorted a[0..n) that are < x (one lane)
__device__ __forceinline__ int lower_bound(const uint64_t* a, int n, uint64_t x) {
  int lo = 0, hi = n;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (a[mid] < x) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// The same count for a warp-uniform x, two shared loads and two ballots for
// n <= 1024: sample every ceil(n/32)-th element, then scan inside the gap.
__device__ __forceinline__ int warp_rank(const uint64_t* a, int n, uint64_t x, int lane) {
  if (n <= 0) return 0;
  if (n > 1024) {
    int r = 0;
    for (int base = 0; base < n; base += 32) {
      const int i = base + lane;
      const unsigned b = __ballot_sync(kFull, i < n && a[i] < x);
      r += __popc(b);
      if (b != kFull) break;
    }
    return r;
  }
  const int step = (n + 31) >> 5;
  const int i = lane * step;
  const int c = __popc(__ballot_sync(kFull, i < n && a[i] < x));
  if (c == 0) return 0;
  const int lo = (c - 1) * step;
  const int j = lo + 1 + lane;
  return lo + 1 + __popc(__ballot_sync(kFull, lane < step - 1 && j < n && a[j] < x));
}

// Merge sorted b[0..m) into sorted a[0..n) in place (keys unique), keeping
// the smallest `cap`.  Returns the new size.  Whole warp, uniform arguments.
__device__ __forceinline__ int warp_merge(uint64_t* a, int n, int cap, const uint64_t* b, int m, int lane) {
  if (m == 0) return n;
  // rb (lane j < m): insertion rank of b_j in a
  int rb = 0;
  if (m <= 4) {
    for (int j = 0; j < m; ++j) {
      const int r = warp_rank(a, n, b[j], lane);
      if (lane == j) rb = r;
    }
  } else if (lane < m) {
    rb = lower_bound(a, n, b[lane]);
  }
  const int p0 = __shfl_sync(kFull, rb, 0);
  // a[i] moves up by #{j : rb_j <= i}; top chunks first so nothing unread is overwritten
  for (int top = n; top > p0; top -= 32) {
    const int i = top - 32 + lane;
    const bool live = i >= p0 && i < n;
    uint64_t x = 0;
    if (live) x = a[i];
    int sh = 0;
    if (m <= 8) {
      for (int j = 0; j < m; ++j) sh += __shfl_sync(kFull, rb, j) <= i ? 1 : 0;
    } else if (live) {
      sh = lower_bound(b, m, x);
    }
    __syncwarp();
    if (live && i + sh < cap) a[i + sh] = x;
    __syncwarp();
  }
  if (lane < m && rb + lane < cap) a[rb + lane] = b[lane];
  __syncwarp();
  const int t = n + m;
  return t < cap ? t : cap;
}

// Bitonic sort of a[0..p2) (p2 a power of two) by one warp.
__device__ inline void warp_bitonic(uint64_t* a, int p2, int lane) {
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
// NB >= 0 fixes the layout at compile time; NB < 0 reads it from nb / nt.
// ---------------------------------------------------------------------------
template <int NB, int NT, int S>
struct Layout {
  int nb_rt, nt_rt;
  __device__ __forceinline__ int nb() const { return NB >= 0 ? NB : nb_rt; }
  __device__ __forceinline__ int nt() const { return NB >= 0 ? NT : nt_rt; }
  __device__ __forceinline__ int elem(int i, int lane) const {
    if (i < nb()) return 64 * i + lane;
    if (i < 2 * nb()) return 64 * (i - nb()) + 32 + lane;
    const int u = i - 2 * nb();
    if (u < nt() && lane < 16) return 64 * nb() + 16 * u + lane;
    return -1;
  }
};

template <int NB, int NT, int S, bool L2>
__device__ __forceinline__ float combine(const Layout<NB, NT, S>& L, const float (&x)[S], const float (&qr)[S]) {
  float a = 0.0f, b = 0.0f;
#pragma unroll
  for (int i = 0; i < S; ++i) {
    if (i < L.nb()) {
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
    if (i >= L.nb() && i < 2 * L.nb()) {
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
    if (i >= 2 * L.nb() && i < 2 * L.nb() + L.nt()) {  // lanes >= 16 hold zeros here
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

// The per-lane chains of one row: a = acc0 (lanes < 16) / acc1 (lanes >= 16),
// b = acc2 / acc3 (the first half of combine()).
template <int NB, int NT, int S, bool L2>
__device__ __forceinline__ void chains(const Layout<NB, NT, S>& L, const float (&x)[S], const float (&qr)[S],
                                       float& a, float& b) {
  a = 0.0f;
  b = 0.0f;
#pragma unroll
  for (int i = 0; i < S; ++i) {
    if (i < L.nb()) {
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
    if (i >= L.nb() && i < 2 * L.nb()) {
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
    if (i >= 2 * L.nb() && i < 2 * L.nb() + L.nt()) {  // lanes >= 16 hold zeros here
      if (L2) {
        const float d = __fsub_rn(qr[i], x[i]);
        a = __fmaf_rn(d, d, a);
      } else {
        a = __fmaf_rn(qr[i], x[i], a);
      }
    }
  }
}

// (acc0 + acc1) + (acc2 + acc3) of two rows with one exchange per sum: lanes
// < 16 finish row 0, lanes >= 16 row 1 (each lane's 16-lane position l =
// lane & 15).  Float addition is commutative, so each sum is bit-identical to
// combine()'s.
__device__ __forceinline__ float pair_sums(float a0, float b0, float a1, float b1, int lane) {
  const bool hi = lane >= 16;
  const float ra = __shfl_xor_sync(kFull, hi ? a0 : a1, 16);
  const float rb = __shfl_xor_sync(kFull, hi ? b0 : b1, 16);
  const float xa = hi ? __fadd_rn(ra, a1) : __fadd_rn(a0, ra);
  const float xb = hi ? __fadd_rn(rb, b1) : __fadd_rn(b0, rb);
  return __fadd_rn(xa, xb);
}

// The 16-lane butterfly (8, 4, 2, 1) of four rows at once: p holds rows 0 / 1
// in lanes < 16 / >= 16, r rows 2 / 3; after the 8-step each 8-lane group
// holds one row (lanes 0-7 row 0, 8-15 row 2, 16-23 row 1, 24-31 row 3).
__device__ __forceinline__ float quad_reduce(float p, float r, int lane) {
  const bool up = (lane & 8) != 0;
  const float rv = __shfl_xor_sync(kFull, up ? p : r, 8);
  float v = up ? __fadd_rn(r, rv) : __fadd_rn(p, rv);
  v = __fadd_rn(v, __shfl_xor_sync(kFull, v, 4));
  v = __fadd_rn(v, __shfl_xor_sync(kFull, v, 2));
  v = __fadd_rn(v, __shfl_xor_sync(kFull, v, 1));
  return v;
}

// Distances for the lanes in `mask`, G rows in flight; lane j receives the
// distance of its own id.  All loads of a group are issued before any math.
template <int NB, int NT, int S, int G, bool L2>
__device__ __forceinline__ float lane_dists(const Layout<NB, NT, S>& L, const float* __restrict__ vecs, uint32_t pd,
                                            uint32_t id, uint32_t mask, const float (&qr)[S], int lane) {
  float mine = 0.0f;
  while (mask) {
    int gl[G];
    const float* rows[G];
#pragma unroll
    for (int g = 0; g < G; ++g) {
      gl[g] = mask ? __ffs(mask) - 1 : -1;
      if (mask) mask &= mask - 1;
      const uint32_t gid = __shfl_sync(kFull, id, gl[g] < 0 ? 0 : gl[g]);
      rows[g] = gl[g] < 0 ? nullptr : vecs + static_cast<size_t>(gid) * pd;
    }
    float x[G][S];
#pragma unroll
    for (int g = 0; g < G; ++g) {
#pragma unroll
      for (int i = 0; i < S; ++i) {
        const int e = L.elem(i, lane);
        x[g][i] = (rows[g] != nullptr && e >= 0) ? __ldg(rows[g] + e) : 0.0f;
      }
    }
    if constexpr (G % 4 == 0) {
      // four rows per reduction: 2.25 shuffles per row instead of 6
#pragma unroll
      for (int g0 = 0; g0 < G; g0 += 4) {
        if (gl[g0] < 0) break;  // warp-uniform: rows fill in order
        float a[4], b[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) chains<NB, NT, S, L2>(L, x[g0 + j], qr, a[j], b[j]);
        const float p = pair_sums(a[0], b[0], a[1], b[1], lane);
        const float r = pair_sums(a[2], b[2], a[3], b[3], lane);
        float v = quad_reduce(p, r, lane);
        if (!L2) v = __fsub_rn(1.0f, v);
        // row j of the group sits in lanes 8 * {0, 2, 1, 3}[j] ..
        int src = -1;
#pragma unroll
        for (int j = 0; j < 4; ++j)
          if (gl[g0 + j] == lane) src = 8 * ((j & 1) * 2 + (j >> 1));
        const float got = __shfl_sync(kFull, v, src < 0 ? 0 : src);
        if (src >= 0) mine = got;
      }
    } else if constexpr (G == 2) {
      // two rows per reduction: 3.5 shuffles per row instead of 6
      if (gl[0] >= 0) {
        float a[2], b[2];
#pragma unroll
        for (int j = 0; j < 2; ++j) chains<NB, NT, S, L2>(L, x[j], qr, a[j], b[j]);
        float v = pair_sums(a[0], b[0], a[1], b[1], lane);  // lanes < 16 row 0, >= 16 row 1
        v = __fadd_rn(v, __shfl_xor_sync(kFull, v, 8));
        v = __fadd_rn(v, __shfl_xor_sync(kFull, v, 4));
        v = __fadd_rn(v, __shfl_xor_sync(kFull, v, 2));
        v = __fadd_rn(v, __shfl_xor_sync(kFull, v, 1));
        if (!L2) v = __fsub_rn(1.0f, v);
        const int src = gl[0] == lane ? 0 : (gl[1] == lane ? 16 : -1);
        const float got = __shfl_sync(kFull, v, src < 0 ? 0 : src);
        if (src >= 0) mine = got;
      }
    } else {
#pragma unroll
      for (int g = 0; g < G; ++g) {
        if (gl[g] >= 0) {  // warp-uniform
          const float d = combine<NB, NT, S, L2>(L, x[g], qr);
          if (gl[g] == lane) mine = d;
        }
      }
    }
  }
  return mine;
}

// ---------------------------------------------------------------------------
// distance policies.  ExactDist: FP32 rows in the reference's AVX-512 order
// (bit-identical distances).  ApproxDist: FP16 or per-row-scaled FP8 E4M3
// rows, FP32 accumulation in any order; RPP rows per warp pass, each row
// spread over 32/RPP lanes holding E consecutive elements (16-byte loads).
// ---------------------------------------------------------------------------
template <int NB, int NT, int S, int G>
struct ExactDist {
  static constexpr bool kApprox = false;
  static constexpr int kMinBlocks = S >= 16 ? 4 : 6;  // (128, 7) measured 9% slower
  Layout<NB, NT, S> L;
  float qr[S];
  __device__ __forceinline__ void setup(uint32_t pd) {
    L.nb_rt = static_cast<int>(pd / 64);
    L.nt_rt = static_cast<int>((pd % 64) / 16);
  }
  // the prepared query (cosine: scaled by inv) in this lane's slots
  __device__ __forceinline__ void load_raw(const float* raw, uint32_t dim, float inv, bool cosine, int lane) {
#pragma unroll
    for (int i = 0; i < S; ++i) {
      const int e = L.elem(i, lane);
      const float v = (e >= 0 && e < static_cast<int>(dim)) ? __ldg(raw + e) : 0.0f;
      qr[i] = cosine ? __fmul_rn(v, inv) : v;
    }
  }
  template <bool L2>
  __device__ __forceinline__ float rows(const float* __restrict__ vecs, uint32_t pd, uint32_t id, uint32_t mask,
                                        int lane) const {
    return lane_dists<NB, NT, S, G, L2>(L, vecs, pd, id, mask, qr, lane);
  }
  __device__ __forceinline__ void init(const SearchParams& P) { setup(P.pd); }
  __device__ __forceinline__ void load_query(const SearchParams& P, const float* raw, const float* inv_norm,
                                             uint32_t q, int lane) {
    load_raw(raw, P.dim, inv_norm ? inv_norm[q] : 1.0f, inv_norm != nullptr, lane);
  }
  template <bool L2>
  __device__ __forceinline__ float dists(const SearchParams& P, uint32_t id, uint32_t mask, int lane) const {
    return rows<L2>(P.vecs, P.pd, id, mask, lane);
  }
};

// ---------------------------------------------------------------------------
// distances in the NEON kernel's order (src/kernels_neon.cpp:10-54): four
// 4-lane accumulators over 16-float blocks, so element 16 i + 4 a + b feeds
// accumulator a, lane b, as a fused chain over i; then (acc0 + acc1) +
// (acc2 + acc3) per lane and vaddvq_f32's (v0 + v1) + (v2 + v3).  (The
// 4-float and scalar tails never run: rows are padded to 16 floats.)  On a
// warp, lane c of each half-warp runs chain c = 4 a + b of one row, so a pass
// computes two rows; the sums are a 4 / 8 / 1 / 2 xor butterfly inside the
// half.  NC > 0 fixes the chain length (pd / 16) at compile time, NC < 0
// reads it at run time with -NC slots; G rows are in flight.  QREG: the
// query's chain elements live in registers (chains up to 32); otherwise
// they are re-read from the query row, which stays in L1.
// ---------------------------------------------------------------------------
template <int NC, int G, bool QREG = true>
struct NeonDist {
  static_assert(G % 2 == 0, "rows go in pairs, one per half-warp");
  static constexpr bool kApprox = false;
  static constexpr int kSlots = NC > 0 ? NC : -NC;
  static constexpr int kMinBlocks = kSlots > 8 ? 4 : 6;
  int nc_rt;
  float qr[QREG ? kSlots : 1];
  const float* qraw;
  uint32_t qdim;
  float qinv;
  bool qcos;
  __device__ __forceinline__ int nc() const { return NC > 0 ? NC : nc_rt; }
  __device__ __forceinline__ void setup(uint32_t pd) { nc_rt = static_cast<int>(pd / 16); }
  __device__ __forceinline__ void load_raw(const float* raw, uint32_t dim, float inv, bool cosine, int lane) {
    qraw = raw;
    qdim = dim;
    qinv = inv;
    qcos = cosine;
    if (QREG) {
      const int c = lane & 15;
#pragma unroll
      for (int i = 0; i < kSlots; ++i) qr[QREG ? i : 0] = qelem(16 * i + c, i);
    }
  }
  __device__ __forceinline__ float qelem(int e, int i) const {
    if (i >= nc() || e >= static_cast<int>(qdim)) return 0.0f;
    const float v = __ldg(qraw + e);
    return qcos ? __fmul_rn(v, qinv) : v;
  }
  template <bool L2>
  __device__ __forceinline__ float rows(const float* __restrict__ vecs, uint32_t pd, uint32_t id, uint32_t mask,
                                        int lane) const {
    constexpr int S = kSlots;
    const int c = lane & 15;
    const int half = lane >> 4;
    float mine = 0.0f;
    while (mask) {
      int gl[G];
#pragma unroll
      for (int g = 0; g < G; ++g) {
        gl[g] = mask ? __ffs(mask) - 1 : -1;
        if (mask) mask &= mask - 1;
      }
      const float* rp[G / 2];
#pragma unroll
      for (int p = 0; p < G / 2; ++p) {
        const int src = gl[2 * p + half];  // this half-warp's row of pass p
        const uint32_t rid = __shfl_sync(kFull, id, src < 0 ? 0 : src);
        rp[p] = src < 0 ? nullptr : vecs + static_cast<size_t>(rid) * pd;
      }
      float x[G / 2][S];
#pragma unroll
      for (int p = 0; p < G / 2; ++p)
#pragma unroll
        for (int i = 0; i < S; ++i) x[p][i] = (rp[p] != nullptr && i < nc()) ? __ldg(rp[p] + 16 * i + c) : 0.0f;
#pragma unroll
      for (int p = 0; p < G / 2; ++p) {
        if (gl[2 * p] < 0) break;  // warp-uniform: rows fill in order
        float acc = 0.0f;
#pragma unroll
        for (int i = 0; i < S; ++i) {
          if (i < nc()) {
            const float qv = QREG ? qr[QREG ? i : 0] : qelem(16 * i + c, i);
            if (L2) {
              const float d = __fsub_rn(qv, x[p][i]);
              acc = __fmaf_rn(d, d, acc);
            } else {
              acc = __fmaf_rn(qv, x[p][i], acc);
            }
          }
        }
        acc = __fadd_rn(acc, __shfl_xor_sync(kFull, acc, 4));  // acc0+acc1 | acc2+acc3
        acc = __fadd_rn(acc, __shfl_xor_sync(kFull, acc, 8));  // v[b]
        acc = __fadd_rn(acc, __shfl_xor_sync(kFull, acc, 1));  // v0+v1 | v2+v3
        acc = __fadd_rn(acc, __shfl_xor_sync(kFull, acc, 2));  // (v0+v1)+(v2+v3)
        if (!L2) acc = __fsub_rn(1.0f, acc);
        const float r0 = __shfl_sync(kFull, acc, 0), r1 = __shfl_sync(kFull, acc, 16);
        if (gl[2 * p] == lane) mine = r0;
        if (gl[2 * p + 1] == lane) mine = r1;
      }
    }
    return mine;
  }
  __device__ __forceinline__ void init(const SearchParams& P) { setup(P.pd); }
  __device__ __forceinline__ void load_query(const SearchParams& P, const float* raw, const float* inv_norm,
                                             uint32_t q, int lane) {
    load_raw(raw, P.dim, inv_norm ? inv_norm[q] : 1.0f, inv_norm != nullptr, lane);
  }
  template <bool L2>
  __device__ __forceinline__ float dists(const SearchParams& P, uint32_t id, uint32_t mask, int lane) const {
    return rows<L2>(P.vecs, P.pd, id, mask, lane);
  }
};

template <int PREC, bool L2, int E>
__device__ __forceinline__ float approx_partial(const SearchParams& P, uint32_t id, int sub, const float (&qa)[E]) {
  float acc = 0.0f;
  if (PREC == 1) {
    const uint4* p = reinterpret_cast<const uint4*>(static_cast<const __half*>(P.vq) +
                                                    static_cast<size_t>(id) * P.pdc + sub * E);
#pragma unroll
    for (int c = 0; c < E / 8; ++c) {
      const uint4 u = __ldg(p + c);
      const uint32_t wds[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
      for (int h = 0; h < 4; ++h) {
        const float2 f = __half22float2(*reinterpret_cast<const __half2*>(&wds[h]));
        const float x0 = f.x, x1 = f.y;
        const float q0 = qa[c * 8 + 2 * h], q1 = qa[c * 8 + 2 * h + 1];
        if (L2) {
          const float d0 = q0 - x0, d1 = q1 - x1;
          acc = __fmaf_rn(d0, d0, acc);
          acc = __fmaf_rn(d1, d1, acc);
        } else {
          acc = __fmaf_rn(q0, x0, acc);
          acc = __fmaf_rn(q1, x1, acc);
        }
      }
    }
  } else {
    const uint4* p = reinterpret_cast<const uint4*>(static_cast<const uint8_t*>(P.vq) +
                                                    static_cast<size_t>(id) * P.pdc + sub * E);
    const float sc = __ldg(P.vscale + id);
#pragma unroll
    for (int c = 0; c < E / 16; ++c) {
      const uint4 u = __ldg(p + c);
      const uint32_t wds[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
      for (int h = 0; h < 4; ++h) {
#pragma unroll
        for (int pr = 0; pr < 2; ++pr) {
          const __nv_fp8x2_storage_t two = static_cast<__nv_fp8x2_storage_t>((wds[h] >> (16 * pr)) & 0xFFFFu);
          const __half2_raw hr = __nv_cvt_fp8x2_to_halfraw2(two, __NV_E4M3);
          const float2 f = __half22float2(*reinterpret_cast<const __half2*>(&hr));
          const float x0 = f.x * sc, x1 = f.y * sc;
          const float q0 = qa[c * 16 + 4 * h + 2 * pr], q1 = qa[c * 16 + 4 * h + 2 * pr + 1];
          if (L2) {
            const float d0 = q0 - x0, d1 = q1 - x1;
            acc = __fmaf_rn(d0, d0, acc);
            acc = __fmaf_rn(d1, d1, acc);
          } else {
            acc = __fmaf_rn(q0, x0, acc);
            acc = __fmaf_rn(q1, x1, acc);
          }
        }
      }
    }
  }
  return acc;
}

// The exact FP32 policy (the index's summation order, runtime lengths) of a
// compressed padded-width class pdc: ORD 0 the AVX-512 order, 1 the NEON order.
template <int PDC, int ORD>
struct ExactFor {
  using type = ExactDist<-1, 0, PDC == 128 ? 5 : (PDC == 256 ? 9 : (PDC == 512 ? 17 : 33)),
                         PDC == 128 ? 4 : (PDC <= 512 ? 2 : 1)>;
};
template <int PDC>
struct ExactFor<PDC, 1> {
  using type = NeonDist<-(PDC <= 512 ? PDC / 16 : 64), PDC == 128 ? 4 : 2, (PDC <= 512)>;
};

template <int RPP, int E, int PREC, int ORD = 0>
struct ApproxDist {
  static constexpr bool kApprox = true;
  static constexpr int kMinBlocks = 5;  // (128, 6) measured 8% slower on the 1M FP8 walk
  static constexpr int LPR = 32 / RPP;
  // the exact FP32 policy of the same padded-width class: the fused rerank
  // computes the pool's exact distances
  static constexpr int kPdc = LPR * E;
  using Exact = typename ExactFor<kPdc, ORD>::type;
  float qa[E];
  __device__ __forceinline__ void init(const SearchParams&) {}
  __device__ __forceinline__ void load_query(const SearchParams& P, const float* raw, const float* inv_norm,
                                             uint32_t q, int lane) {
    const float inv = inv_norm ? inv_norm[q] : 1.0f;
    const int base = (lane % LPR) * E;
#pragma unroll
    for (int e = 0; e < E; ++e) {
      // the copy stores rows in the tensor-core order (compressed_layout.cuh)
      const int idx = static_cast<int>(cl_logical(static_cast<uint32_t>(base + e), PREC));
      const float v = idx < static_cast<int>(P.dim) ? __ldg(raw + idx) : 0.0f;
      qa[e] = inv_norm ? __fmul_rn(v, inv) : v;
    }
  }
  template <bool L2>
  __device__ __forceinline__ float dists(const SearchParams& P, uint32_t id, uint32_t mask, int lane) const {
    const int qi = lane / LPR, sub = lane % LPR;
    float mine = 0.0f;
    while (mask) {
      int ow[RPP];
      uint32_t rid[RPP];
#pragma unroll
      for (int r = 0; r < RPP; ++r) {
        ow[r] = mask ? __ffs(mask) - 1 : -1;
        if (mask) mask &= mask - 1;
        rid[r] = __shfl_sync(kFull, id, ow[r] < 0 ? 0 : ow[r]);
      }
      int myow = ow[0];
      uint32_t myid = rid[0];
#pragma unroll
      for (int r = 1; r < RPP; ++r)
        if (qi == r) {
          myow = ow[r];
          myid = rid[r];
        }
      float acc = myow >= 0 ? approx_partial<PREC, L2, E>(P, myid, sub, qa) : 0.0f;
#pragma unroll
      for (int o = LPR / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(kFull, acc, o);
#pragma unroll
      for (int r = 0; r < RPP; ++r) {
        const float v = __shfl_sync(kFull, acc, r * LPR);
        if (ow[r] == lane) mine = L2 ? v : 1.0f - v;
      }
    }
    return mine;
  }
};

// ---------------------------------------------------------------------------
// per-warp state
// ---------------------------------------------------------------------------
// The warp's shared-memory slab is [hash: H u32][res: R keys][cand: C + 32
// keys][stA: 32][stE: 32]; the parts are derived from its base and the
// launch's H / R / C (constant bank) rather than kept in registers.
// Per-warp state written by every lane with the same value (so each lane
// reads back a value it wrote itself) or by lane 0 alone for the counters.
struct WarpCold {
  uint64_t* pool;        // spill pool in use (null until the first spill)
  const uint32_t* fb;    // the query's filter bits or null
  int pool_idx;          // acquired shared pool (-1 none)
  int big_idx;           // acquired second-tier pool (-1 none)
  int bm_idx;            // acquired shared bitmap (-1 none)
  uint32_t peak;         // largest head + pool size seen
  uint32_t n_lists;      // layer-0 lists read (counters only)
  uint32_t n_dists;      // layer-0 distances (counters only)
  uint32_t spilled;      // the candidate pool was used
};
static_assert(sizeof(WarpCold) <= 64, "the warp's shared region reserves 64 bytes for WarpCold");

// global warp slot (fixed scratch of the non-shared layouts; acquire's start)
__device__ __forceinline__ uint64_t warp_slot(const SearchParams& P) {
  return P.slot_base + static_cast<uint64_t>(blockIdx.x) * (blockDim.x >> 5) + (threadIdx.x >> 5);
}

struct Warp {
  unsigned char* base;
  __device__ __forceinline__ uint32_t* hash() const { return reinterpret_cast<uint32_t*>(base); }
  __device__ __forceinline__ uint64_t* res(const SearchParams& P) const {
    return reinterpret_cast<uint64_t*>(base + 4u * P.H);
  }
  __device__ __forceinline__ uint64_t* cand(const SearchParams& P) const { return res(P) + P.R; }
  __device__ __forceinline__ uint64_t* stA(const SearchParams& P) const { return cand(P) + P.C + 32; }
  __device__ __forceinline__ uint64_t* stE(const SearchParams& P) const { return stA(P) + 32; }
  // state the traversal loop rarely touches lives in shared memory, not registers
  __device__ __forceinline__ WarpCold* cold(const SearchParams& P) const {
    return reinterpret_cast<WarpCold*>(stE(P) + 32);
  }
  uint32_t* bitmap;   // visited bitmap in use
  uint32_t tag;       // epoch << 24 (tagged mode)
  uint32_t vcount;    // visited entries in the hash
  bool bitmap_mode;
};

// Claim a free entry of a shared scratch array: one bounded pass over the
// owner flags from a slot-dependent start, 32 flags per step (never waits).
// -1 if all are taken.
__device__ __forceinline__ int acquire(uint32_t* owner, uint32_t nslots, uint64_t slot, int lane) {
  const uint32_t start = static_cast<uint32_t>((slot * 2654435761ull) % nslots);
  for (uint32_t t = 0; t < nslots; t += 32) {
    uint32_t i = start + t + static_cast<uint32_t>(lane);
    if (i >= nslots) i -= nslots;
    const bool open = t + static_cast<uint32_t>(lane) < nslots &&
                      *reinterpret_cast<volatile const uint32_t*>(owner + i) == 0u;
    uint32_t b = __ballot_sync(kFull, open);
    while (b) {
      const int l = __ffs(b) - 1;
      b &= b - 1;
      int got = 0;
      if (lane == l) got = atomicCAS(owner + i, 0u, 1u) == 0u;
      if (__shfl_sync(kFull, got, l)) return static_cast<int>(__shfl_sync(kFull, i, l));
    }
  }
  return -1;
}

// Give back the shared scratch a query held (its writes are complete first).
__device__ __forceinline__ void release_scratch(Warp& w, const SearchParams& P, int lane) {
  __syncwarp();
  __threadfence();
  WarpCold* cw = w.cold(P);
  if (lane == 0) {
    if (cw->pool_idx >= 0) atomicExch(P.pool_owner + cw->pool_idx, 0u);
    if (cw->big_idx >= 0) atomicExch(P.big_owner + cw->big_idx, 0u);
    if (cw->bm_idx >= 0) atomicExch(P.bm_owner + cw->bm_idx, 0u);
  }
  __syncwarp();
  cw->pool_idx = -1;
  cw->big_idx = -1;
  cw->bm_idx = -1;
  cw->pool = nullptr;
  __syncwarp();
}

__device__ __forceinline__ bool hash_empty(uint32_t v, uint32_t tag, bool tagged) {
  return tagged ? ((v & 0xFF000000u) != tag) : (v == kNoId);
}

// Test-and-mark `id` (valid lanes only); returns true if it was visited.
__device__ __forceinline__ bool visit(Warp& w, const SearchParams& P, uint32_t id, bool tagged) {
  if (w.bitmap_mode) {
    const uint32_t bit = 1u << (id & 31u);
    const uint32_t old = atomicOr(&w.bitmap[id >> 5], bit);
    return (old & bit) != 0;
  }
  const uint32_t key = tagged ? (w.tag | id) : id;
  uint32_t p = (id * 0x9E3779B1u) >> (1 + __clz(P.H));
  for (;;) {
    const uint32_t v = *reinterpret_cast<volatile const uint32_t*>(&w.hash()[p]);
    if (!hash_empty(v, w.tag, tagged)) {
      if (v == key) return true;
      p = (p + 1) & (P.H - 1u);
      continue;
    }
    const uint32_t old = atomicCAS(&w.hash()[p], v, key);
    if (old == v) return false;
    if (old == key) return true;
  }
}

// Move the visited set from the hash to a bitmap (false: none available).
__device__ __forceinline__ bool to_bitmap(Warp& w, const SearchParams& P, bool tagged, int lane) {
  const uint64_t words = P.bitmap_words;
  if (P.bm_owner) {
    const int i = acquire(P.bm_owner, P.bm_slots, warp_slot(P), lane);
    if (i < 0) return false;
    w.cold(P)->bm_idx = i;
    w.bitmap = P.bitmaps + static_cast<uint64_t>(i) * words;
  } else {
    w.bitmap = P.bitmaps + warp_slot(P) * words;
  }
  for (uint64_t i = lane; i < words; i += 32) w.bitmap[i] = 0u;
  __syncwarp();
  for (uint32_t p = lane; p <= (P.H - 1u); p += 32) {
    const uint32_t v = w.hash()[p];
    if (!hash_empty(v, w.tag, tagged)) {
      const uint32_t id = tagged ? (v & 0x00FFFFFFu) : v;
      atomicOr(&w.bitmap[id >> 5], 1u << (id & 31u));
    }
  }
  __syncwarp();
  w.bitmap_mode = true;
  return true;
}

__device__ __forceinline__ bool bit_of(const uint32_t* bits, uint32_t id) {
  return ((__ldg(bits + (id >> 5)) >> (id & 31u)) & 1u) != 0;
}

// Radix select: the r-th smallest (1-based) of pool[0..pn).  hist: 256 u32 in smem.
__device__ inline uint64_t radix_select(const uint64_t* pool, uint64_t pn, uint64_t r, uint32_t* hist, int lane) {
  uint64_t prefix = 0, pmask = 0;
  for (int shift = 56; shift >= 0; shift -= 8) {
    for (int i = lane; i < 256; i += 32) hist[i] = 0u;
    __syncwarp();
    for (uint64_t i = lane; i < pn; i += 32) {
      const uint64_t x = pool[i];
      if ((x & pmask) == prefix) atomicAdd(&hist[(x >> shift) & 255u], 1u);
    }
    __syncwarp();
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
    const int owner = __ffs(__ballot_sync(kFull, here)) - 1;
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
  uint32_t pn;    // pool entries (at most the second tier's capacity)
  uint64_t pmin;  // min key in pool (kMaxKey if empty)
  bool overflow;
};

// Move a pool of pn keys to the second tier (capacity big_cap); returns the
// entry taken or -1.  Holders of second-tier entries wait on nothing, so the
// bounded wait for a free entry ends; past the bound the query goes to the
// rerun pass.  Plain arguments keep the caller's state in registers.
static __device__ __noinline__ int promote_pool(uint64_t* big_pool, uint64_t big_cap, uint32_t* big_owner,
                                                uint32_t big_slots, const uint64_t* src, uint64_t pn, uint64_t slot,
                                                int lane) {
  int i = -1;
  for (uint32_t tries = 0; tries < kBigPoolTries; ++tries) {
    i = acquire(big_owner, big_slots, slot, lane);
    if (i >= 0) break;
    __nanosleep(2000);
  }
  if (i < 0) return -1;
  uint64_t* big = big_pool + static_cast<uint64_t>(i) * big_cap;
  for (uint64_t j = lane; j < pn; j += 32) big[j] = src[j];
  __syncwarp();
  __threadfence();
  return i;
}

__device__ __forceinline__ bool pool_append(Warp& w, Cands& c, const SearchParams& P, const uint64_t* src, int cnt,
                                            int lane) {
  if (cnt <= 0) return true;
  WarpCold* cw = w.cold(P);
  uint64_t* pool = cw->pool;
  const int big_idx = cw->big_idx;
  const uint64_t cap = big_idx >= 0 ? P.big_cap : P.pool_cap;
  if (c.pn + static_cast<uint64_t>(cnt) > cap) {
    const int i = (big_idx >= 0 || P.big_owner == nullptr || c.pn + static_cast<uint64_t>(cnt) > P.big_cap ||
                   pool == nullptr)
                      ? -1
                      : promote_pool(P.big_pool, P.big_cap, P.big_owner, P.big_slots, pool, c.pn, warp_slot(P), lane);
    if (i < 0) {
      c.overflow = true;
      return false;
    }
    if (lane == 0 && cw->pool_idx >= 0) atomicExch(P.pool_owner + cw->pool_idx, 0u);
    __syncwarp();
    pool = P.big_pool + static_cast<uint64_t>(i) * P.big_cap;
    cw->pool_idx = -1;
    cw->big_idx = i;
    cw->pool = pool;
  }
  if (pool == nullptr) {
    if (P.pool_owner) {
      const int i = acquire(P.pool_owner, P.pool_slots, warp_slot(P), lane);
      if (i < 0) {
        c.overflow = true;
        return false;
      }
      cw->pool_idx = i;
      pool = P.pool + static_cast<uint64_t>(i) * P.pool_cap;
    } else {
      pool = P.pool + warp_slot(P) * P.pool_cap;
    }
    cw->pool = pool;
  }
  if (lane < cnt) pool[c.pn + lane] = src[lane];
  c.pn += cnt;
  cw->spilled = 1u;
  return true;
}

// Merge a register buffer (one key per lane, lanes in `valid`) into the sorted
// array a[0..n) of capacity cap through the staging array st; returns the new
// length.  Out of line: it runs once per 32 accepted results.
static __device__ __noinline__ int merge_buffer(uint64_t key, uint32_t valid, uint64_t* a, int n, int cap, uint64_t* st,
                                                int lane) {
  const uint64_t v = warp_sort32(((valid >> lane) & 1u) ? key : kMaxKey, lane);
  const int m = __popc(valid);
  if (lane < m) st[lane] = v;
  __syncwarp();
  return warp_merge(a, n, cap, st, m, lane);
}

// Refill an empty head from the pool with its smallest keys (at most C/2);
// when the result set is full, first drop pool keys farther than the worst.
// Out of line with plain arguments: a rare path kept out of the traversal
// loop's instruction footprint.
struct RefillOut {
  int ct;
  uint32_t pn;
  uint64_t pmin;
};
static __device__ __noinline__ RefillOut refill_core(uint64_t* pool, uint32_t pn, uint64_t* cand, uint32_t C,
                                                     bool res_full, float worst_d, int lane) {
  if (res_full) {
    uint64_t wpos = 0;
    for (uint64_t base = 0; base < pn; base += 32) {
      const uint64_t i = base + lane;
      uint64_t x = 0;
      bool keep = false;
      if (i < pn) {
        x = pool[i];
        keep = key_dist(x) <= worst_d;
      }
      const uint32_t bal = __ballot_sync(kFull, keep);
      __syncwarp();
      if (keep) pool[wpos + __popc(bal & ((1u << lane) - 1u))] = x;
      wpos += __popc(bal);
      __syncwarp();
    }
    pn = static_cast<uint32_t>(wpos);
  }
  RefillOut o{0, pn, kMaxKey};
  if (pn == 0) return o;
  const uint64_t half = C / 2;
  const uint64_t take = pn < half ? pn : half;
  uint64_t T = kMaxKey;
  if (pn > take) T = radix_select(pool, pn, take, reinterpret_cast<uint32_t*>(cand), lane);
  __syncwarp();
  uint64_t hpos = 0, wpos = 0, newmin = kMaxKey;
  for (uint64_t base = 0; base < pn; base += 32) {
    const uint64_t i = base + lane;
    uint64_t x = kMaxKey;
    const bool live = i < pn;
    if (live) x = pool[i];
    const bool sel = live && x <= T;
    const bool rest = live && !sel;
    const uint32_t bs = __ballot_sync(kFull, sel);
    const uint32_t br = __ballot_sync(kFull, rest);
    __syncwarp();
    const uint32_t below = (1u << lane) - 1u;
    if (sel) cand[hpos + __popc(bs & below)] = x;
    if (rest) {
      pool[wpos + __popc(br & below)] = x;
      newmin = x < newmin ? x : newmin;
    }
    hpos += __popc(bs);
    wpos += __popc(br);
    __syncwarp();
  }
  newmin = ~warp_max64(~newmin);
  int p2 = 1;
  while (p2 < static_cast<int>(hpos)) p2 <<= 1;
  for (int i = static_cast<int>(hpos) + lane; i < p2; i += 32) cand[i] = kMaxKey;
  __syncwarp();
  warp_bitonic(cand, p2, lane);
  o.ct = static_cast<int>(hpos);
  o.pn = static_cast<uint32_t>(wpos);
  o.pmin = wpos ? newmin : kMaxKey;
  return o;
}

__device__ __forceinline__ void refill(Warp& w, Cands& c, const SearchParams& P, bool res_full, float worst_d, int lane) {
  __syncwarp();
  const RefillOut o = refill_core(w.cold(P)->pool, c.pn, w.cand(P), P.C, res_full, worst_d, lane);
  c.ch = 0;
  c.ct = o.ct;
  c.pn = o.pn;
  c.pmin = o.pmin;
}

// Insert the sorted accepted batch stA[0..m) into the candidate queue.
// Once the result set is full, head keys farther than the worst result are
// dropped before anything would spill to the pool.
__device__ __forceinline__ void cand_insert(Warp& w, Cands& c, const SearchParams& P, int m, bool res_full, float worst_d,
                            int lane) {
  if (m <= 0) return;
  const int C = static_cast<int>(P.C);
  if (res_full && c.ct + m > C) {
    int lo = c.ch, hi = c.ct;  // first head key farther than the worst result
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (key_dist(w.cand(P)[mid]) > worst_d) hi = mid;
      else lo = mid + 1;
    }
    c.ct = lo;
  }
  int mh = m;
  if (c.pn > 0) {
    mh = __popc(__ballot_sync(kFull, lane < m && w.stA(P)[lane] < c.pmin));
    if (m > mh && !pool_append(w, c, P, w.stA(P) + mh, m - mh, lane)) return;
  }
  if (mh > 0) {
    const int n = c.ct - c.ch;
    const int nn = warp_merge(w.cand(P) + c.ch, n, C + 32 - c.ch, w.stA(P), mh, lane);
    c.ct = c.ch + nn;
    if (c.ct > C) {
      if (c.ch > 0) {  // compact to the front
        const int len = c.ct - c.ch;
        for (int base = 0; base < len; base += 32) {
          const int i = base + lane;
          uint64_t x = 0;
          if (i < len) x = w.cand(P)[c.ch + i];
          __syncwarp();
          if (i < len) w.cand(P)[i] = x;
          __syncwarp();
        }
        c.ct = len;
        c.ch = 0;
      }
      if (c.ct > C) {  // spill the largest keys
        const int cnt = c.ct - C;
        const uint64_t first = w.cand(P)[C];
        if (!pool_append(w, c, P, w.cand(P) + C, cnt, lane)) return;
        c.pmin = first < c.pmin ? first : c.pmin;
        c.ct = C;
      }
    }
  }
  if (P.counters) {
    WarpCold* cw = w.cold(P);
    const uint32_t total = static_cast<uint32_t>(c.ct - c.ch) + static_cast<uint32_t>(c.pn);
    cw->peak = total > cw->peak ? total : cw->peak;
  }
}

// Publish query q's output row: every lane's writes are fenced at system
// scope before lane 0 raises the flag, so a host thread that sees the flag
// (acquire) sees the row (the server's per-request completion).
__device__ __forceinline__ void signal_done(uint32_t* done, uint32_t q, int lane) {
  __threadfence_system();
  __syncwarp();
  if (lane == 0) *reinterpret_cast<volatile uint32_t*>(done + q) = 1u;
}

// Exact FP32 distances (reference order, layout EX) of the s pool ids in
// prow, merged 32 at a time into res (sorted, capacity R).  Kept out of line
// with plain arguments: its registers do not add to the traversal loop's.
template <class EX, bool L2>
static __device__ __noinline__ void fused_rerank(const float* __restrict__ vecs, uint32_t pd, uint32_t dim,
                                                 const float* __restrict__ raw, float inv, bool cosine,
                                                 const uint32_t* prow, int s, uint64_t* res, uint64_t* stE, int R,
                                                 int lane) {
  EX ex;
  ex.setup(pd);
  ex.load_raw(raw, dim, inv, cosine, lane);
  int n = 0;
  for (int c0 = 0; c0 < s; c0 += 32) {
    const bool live = c0 + lane < s;
    const uint32_t id = live ? prow[c0 + lane] : kNoId;
    const uint32_t mask = __ballot_sync(kFull, live);
    const float d = ex.template rows<L2>(vecs, pd, id, mask, lane);
    const uint64_t v = warp_sort32(live ? mkkey(d, id) : kMaxKey, lane);
    const int mm = __popc(mask);
    if (lane < mm) stE[lane] = v;
    __syncwarp();
    n = warp_merge(res, n, R, stE, mm, lane);
    __syncwarp();
  }
}

struct QueryOut {
  uint64_t label;
  float dist;
  uint32_t zero;
};

// ---------------------------------------------------------------------------
// the kernel
// ---------------------------------------------------------------------------
template <class DP, bool L2>
__global__ void __launch_bounds__(128, DP::kMinBlocks) search_kernel(SearchParams P, const float* __restrict__ inv_norm) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const uint32_t per_warp = warp_smem_bytes(P.H, P.R, P.C);
  unsigned char* base = smem + static_cast<size_t>(wib) * per_warp;
  Warp w;
  w.base = base;
  w.bitmap = nullptr;
  {
    WarpCold* cw = w.cold(P);
    cw->pool = nullptr;
    cw->pool_idx = -1;
    cw->big_idx = -1;
    cw->bm_idx = -1;
  }
  const bool tagged = P.tagged != 0;
  uint32_t epoch = 0;
  for (uint32_t i = lane; i < P.H; i += 32) w.hash()[i] = tagged ? 0u : kNoId;
  __syncwarp();

  DP dp;
  dp.init(P);
  // a queue length read from the device never exceeds the batch (its list
  // holds at most P.nq entries)
  const bool single_chunk = P.M0 <= 32;
  uint32_t nq = P.nq_dev ? min(*P.nq_dev, P.nq) : P.nq;
  if (P.lpt_sizes) {
    nq = 0;
    for (uint32_t b = 0; b < P.lpt_buckets; ++b) nq += P.lpt_sizes[b];
    nq = min(nq, P.nq);
  }

  for (;;) {
    uint32_t item = 0;
    if (lane == 0) item = atomicAdd(P.work, 1u);
    item = __shfl_sync(kFull, item, 0);
    if (item >= nq) break;
    uint32_t q;
    if (P.lpt_sizes) {  // largest-ef bucket first (longest queries start first)
      uint32_t rem = item;
      uint32_t b = P.lpt_buckets - 1;
      while (b > 0 && rem >= P.lpt_sizes[b]) {
        rem -= P.lpt_sizes[b];
        --b;
      }
      q = P.qidx[static_cast<size_t>(b) * P.lpt_stride + rem];
    } else {
      q = P.qidx ? P.qidx[item] : item;
    }
    if (q >= P.nq) continue;  // list entries are query indices of this batch

    uint32_t k = P.kq ? P.kq[q] : P.k_all;
    uint32_t ef = P.efq ? P.efq[q] : P.ef_all;
    if (ef == 0) ef = P.ef_default;
    if (ef < k) ef = k;
    if (ef > P.R || k > P.k_stride || k == 0) {
      // device-side arrays promised a smaller bound: refuse this query
      if (lane == 0) atomicExch(P.err, 1u);
      continue;
    }
    const int efi = static_cast<int>(ef);
    bool filtered = P.deleted_any != 0;
    {
      const uint32_t* fb = nullptr;
      if (P.fsel) {
        const int32_t f = P.fsel[q];
        if (f >= 0) fb = P.fbits[f];
      }
      filtered = filtered || fb != nullptr;
      WarpCold* cw = w.cold(P);
      cw->fb = fb;
      cw->peak = 0;
      cw->spilled = 0;
      if (lane == 0) {
        cw->n_lists = 0;
        cw->n_dists = 0;
      }
    }
    // traversal counters; the upper-layer ones are stored when the descent
    // ends, the layer-0 ones are kept in shared memory, and nodes visited at
    // layer 0 = distances + the entry point
    uint32_t n_uplists = 0, n_updists = 0;
    bool ran = false;

    int s = 0;  // result count
    Cands c{0, 0, 0u, kMaxKey, false};
    if (P.n > 0) {
      // ---- query registers (prepare_vector: cosine scaled by 1/||q||) ----
      dp.load_query(P, P.queries + static_cast<size_t>(q) * P.dim, inv_norm, q, lane);
      // ---- visited set for this query ----
      w.bitmap_mode = false;
      w.vcount = 0;
      if (tagged) {
        if (++epoch == 256u) {
          for (uint32_t i = lane; i < P.H; i += 32) w.hash()[i] = 0u;
          __syncwarp();
          epoch = 1;
        }
        w.tag = epoch << 24;
      } else {
        for (uint32_t i = lane; i < P.H; i += 32) w.hash()[i] = kNoId;
        __syncwarp();
        w.tag = 0;
      }

      // ---- entry point + greedy descent (search_layer.cpp:29-56,156-157) ----
      uint32_t cur = P.entry;
      float cur_d = dp.template dists<L2>(P, cur, 1u, lane);
      cur_d = __shfl_sync(kFull, cur_d, 0);
      n_updists = 1;
      for (int lc = P.max_level; lc > 0; --lc) {
        bool changed = true;
        while (changed) {
          changed = false;
          const uint32_t* lst = P.up + static_cast<size_t>(__ldg(P.up_blk + cur) + (lc - 1)) * P.up_stride;
          ++n_uplists;
          for (uint32_t c0 = 0; c0 < P.M; c0 += 32) {
            const uint32_t j = c0 + lane;
            const uint32_t id = j < P.M ? __ldg(lst + j) : kNoId;
            const uint32_t vm = __ballot_sync(kFull, id != kNoId);
            if (!vm) break;
            n_updists += __popc(vm);
            const float d = dp.template dists<L2>(P, id, vm, lane);
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

      if (P.counters && lane == 0) {  // the descent's counters, stored now so they are not kept live
        unsigned long long* cp = P.counters + static_cast<size_t>(q) * kCounters;
        cp[0] = n_uplists;
        cp[1] = n_updists;
      }
      // ---- layer 0 (search_layer.cpp:58-134) ----
      // Results: sorted base res[0..rtop] in shared memory plus up to 32 newly
      // inserted keys in a register buffer (one per lane: rk, live set rvalid,
      // largest rmax).  Candidates: sorted head cand[ch..ct) (+ spill pool)
      // plus a register buffer (ck, cvalid, smallest cmin).  Buffers are
      // merged into the arrays when 32 keys have gathered.
      if (lane == 0) visit(w, P, cur, tagged);
      __syncwarp();
      w.vcount = 1;
      ran = true;
      const uint64_t k0 = mkkey(cur_d, cur);
      const uint32_t* fb0 = w.cold(P)->fb;
      const bool e0 = !filtered || (bit_of(P.alive, cur) && (!fb0 || bit_of(fb0, cur)));
      if (lane == 0) {
        w.cand(P)[0] = k0;
        if (e0) w.res(P)[0] = k0;
      }
      c.ct = 1;
      if (P.counters) w.cold(P)->peak = 1;
      int rtop = e0 ? 0 : -1;
      s = rtop + 1;
      uint64_t rk = kMaxKey, ck = kMaxKey, rmax = 0, cmin = kMaxKey;
      uint32_t rvalid = 0, cvalid = 0;
      float worst_d = (e0 && efi <= 1) ? cur_d : 0.0f;  // distance of the worst result once s >= ef
      __syncwarp();

      // merge the result buffer into the sorted base
      auto flush_res = [&]() {
        rtop = merge_buffer(rk, rvalid, w.res(P), rtop + 1, static_cast<int>(P.R), w.stE(P), lane) - 1;
        rvalid = 0;
        rk = kMaxKey;
        rmax = 0;
      };
      // merge the candidate buffer into the head (dropping keys past the worst result)
      auto flush_cand = [&]() {
        const uint64_t v = warp_sort32(((cvalid >> lane) & 1u) ? ck : kMaxKey, lane);
        const bool full = s >= efi;
        int m = __popc(cvalid);
        if (full) m = __popc(__ballot_sync(kFull, lane < m && key_dist(v) <= worst_d));
        if (lane < m) w.stA(P)[lane] = v;
        __syncwarp();
        cand_insert(w, c, P, m, full, worst_d, lane);
        cvalid = 0;
        ck = kMaxKey;
        cmin = kMaxKey;
      };

      const uint32_t hlimit = (P.H * 5u) / 8u;
      uint32_t pf_cid = kNoId, pf_id = kNoId;  // adjacency of the next candidate, loaded ahead
      for (;;) {
        if (c.ch == c.ct && c.pn > 0) refill(w, c, P, s >= efi, worst_d, lane);
        const uint64_t bh = c.ch < c.ct ? w.cand(P)[c.ch] : kMaxKey;
        const uint64_t top = bh < cmin ? bh : cmin;
        if (top == kMaxKey) break;
        if (s >= efi && key_dist(top) > worst_d) break;
        if (bh < cmin) {
          c.ch++;
        } else {  // the best candidate sits in the register buffer
          cvalid &= ~__ballot_sync(kFull, ((cvalid >> lane) & 1u) && ck == cmin);
          cmin = warp_min64(((cvalid >> lane) & 1u) ? ck : kMaxKey);
        }
        const uint32_t cid = static_cast<uint32_t>(top);
        const uint32_t* lst = P.l0 + static_cast<size_t>(cid) * P.l0_stride;
        if (P.counters && lane == 0) w.cold(P)->n_lists++;
        for (uint32_t c0 = 0; c0 < P.M0; c0 += 32) {
          const uint32_t j = c0 + lane;
          uint32_t id;
          if (c0 == 0 && cid == pf_cid) id = pf_id;
          else id = j < P.M0 ? __ldg(lst + j) : kNoId;
          if (c0 == 0 && single_chunk) {
            // load the list of the next candidate while this one is expanded
            const uint64_t nb = c.ch < c.ct ? w.cand(P)[c.ch] : kMaxKey;
            const uint64_t nx = nb < cmin ? nb : cmin;
            pf_cid = nx != kMaxKey ? static_cast<uint32_t>(nx) : kNoId;
            if (pf_cid != kNoId) pf_id = lane < static_cast<int>(P.M0)
                                             ? __ldg(P.l0 + static_cast<size_t>(pf_cid) * P.l0_stride + lane)
                                             : kNoId;
          }
          const bool valid = id != kNoId;
          const uint32_t vm = __ballot_sync(kFull, valid);
          if (!vm) break;
          if (!w.bitmap_mode && w.vcount + __popc(vm) > hlimit && !to_bitmap(w, P, tagged, lane)) {
            c.overflow = true;  // no bitmap free: the rerun pass answers this query
            break;
          }
          bool first = valid;
          if (P.dedup && valid) {
            const uint32_t same = __match_any_sync(vm, id);
            first = (__ffs(same) - 1) == lane;
          }
          bool fresh = false;
          if (first) fresh = !visit(w, P, id, tagged);
          __syncwarp();
          uint32_t U = __ballot_sync(kFull, fresh);
          const int nu = __popc(U);
          w.vcount += nu;
          if (!U) continue;
          if (P.counters && lane == 0) w.cold(P)->n_dists += nu;
          // eligibility words load while the rows are gathered
          uint32_t ew = ~0u;
          if (filtered && fresh) {
            const uint32_t* fb = w.cold(P)->fb;
            const uint32_t aw = __ldg(P.alive + (id >> 5));
            const uint32_t fw = fb ? __ldg(fb + (id >> 5)) : ~0u;
            ew = aw & fw;
          }
          const float d = dp.template dists<L2>(P, id, U, lane);
          const bool elig = ((ew >> (id & 31u)) & 1u) != 0;
          const uint64_t key = mkkey(d, id);

          // ---- in-order acceptance replay (search_layer.cpp:112-132) ----
          if (s >= efi) U &= __ballot_sync(kFull, d < worst_d);  // the worst only decreases
          while (U) {
            const int jl = __ffs(U) - 1;
            U &= U - 1;
            const float dj = __shfl_sync(kFull, d, jl);
            if (!(s < efi || dj < worst_d)) continue;
            const uint64_t kj = shfl64(key, jl);
            // candidate
            if (cvalid == kFull) {
              flush_cand();
              if (c.overflow) break;
            }
            {
              const int slot = __ffs(~cvalid) - 1;
              if (lane == slot) ck = kj;
              cvalid |= 1u << slot;
              cmin = kj < cmin ? kj : cmin;
            }
            if (!__shfl_sync(kFull, elig, jl)) continue;
            // result
            if (rvalid == kFull) flush_res();
            {
              const int slot = __ffs(~rvalid) - 1;
              if (lane == slot) rk = kj;
              rvalid |= 1u << slot;
              rmax = kj > rmax ? kj : rmax;
            }
            if (s < efi) {
              if (++s < efi) continue;
            } else {  // evict the largest of res[rtop] and the buffer
              const uint64_t bt = rtop >= 0 ? w.res(P)[rtop] : 0ull;
              if (bt > rmax) {
                --rtop;
              } else {
                rvalid &= ~__ballot_sync(kFull, ((rvalid >> lane) & 1u) && rk == rmax);
                rmax = warp_max64(((rvalid >> lane) & 1u) ? rk : 0ull);
              }
            }
            const uint64_t bt = rtop >= 0 ? w.res(P)[rtop] : 0ull;
            worst_d = key_dist(bt > rmax ? bt : rmax);
          }
          if (c.overflow) break;
          if (P.counters) {
            WarpCold* cw = w.cold(P);
            const uint32_t live = static_cast<uint32_t>(c.ct - c.ch) + c.pn + __popc(cvalid);
            cw->peak = live > cw->peak ? live : cw->peak;
          }
        }
        if (c.overflow) break;
      }
      if (!c.overflow) flush_res();  // res[0..s) sorted for the output
    }

    const bool used_bitmap = w.bitmap_mode;
    const bool used_pool2 = w.cold(P)->big_idx >= 0;
    release_scratch(w, P, lane);
    if (c.overflow) {
      if (lane == 0) {
        const uint32_t o = atomicAdd(P.ovf_count, 1u);
        if (o < P.nq) P.ovf_list[o] = q;  // at most one entry per query of the batch
      }
      continue;
    }

    const uint32_t kq = P.kq ? P.kq[q] : P.k_all;  // re-read: not kept live across the walk
    if constexpr (DP::kApprox) {
      // Exact FP32 rerank of the traversal pool, fused: the pool ids go to the
      // query's global row, their distances are recomputed in the reference's
      // order and merged 32 at a time into the (now free) result array.  With
      // a rerank factor only the pool's best factor x k (at least 32) are
      // reranked; the pool is sorted by traversal distance.
      if (P.rerank_factor) {
        const uint64_t depth = max(32ull, static_cast<unsigned long long>(P.rerank_factor) * kq);
        if (static_cast<uint64_t>(s) > depth) s = static_cast<int>(depth);
      }
      uint32_t* prow = P.pool_out + static_cast<size_t>(q) * P.pool_stride;
      for (int j = lane; j < s; j += 32) prow[j] = static_cast<uint32_t>(w.res(P)[j]);
      if (lane == 0) P.pool_n[q] = static_cast<uint32_t>(s);
      __syncwarp();
      fused_rerank<typename DP::Exact, L2>(P.vecs, P.pd, P.dim, P.queries + static_cast<size_t>(q) * P.dim,
                                          inv_norm ? inv_norm[q] : 1.0f, inv_norm != nullptr, prow, s, w.res(P), w.stE(P),
                                          static_cast<int>(P.R), lane);
    }
    // ---- output (search_layer.cpp:166-169, 189-192) ----
    const int m = s < static_cast<int>(kq) ? s : static_cast<int>(kq);
    {
      QueryOut* row = static_cast<QueryOut*>(P.out) + static_cast<size_t>(q) * P.k_stride;
      for (uint32_t j = lane; j < P.k_stride; j += 32) {
        QueryOut o;
        if (static_cast<int>(j) < m) {
          const uint64_t kk = w.res(P)[j];
          o.label = P.labels[static_cast<uint32_t>(kk)];
          o.dist = key_dist(kk);
        } else {
          o.label = ~0ull;
          o.dist = __int_as_float(0x7f800000);
        }
        o.zero = 0;
        row[j] = o;
      }
    }
    if (P.nres && lane == 0) P.nres[q] = static_cast<uint32_t>(m);
    if (P.done) signal_done(P.done, q, lane);
    if (P.counters && lane == 0) {
      const WarpCold* cw = w.cold(P);
      const uint32_t n_lists = cw->n_lists, n_dists = cw->n_dists;
      unsigned long long* cp = P.counters + static_cast<size_t>(q) * kCounters;
      if (!ran) {
        cp[0] = 0;
        cp[1] = 0;
      }
      cp[2] = n_lists;
      cp[3] = n_dists;
      cp[4] = ran ? n_dists + 1u : 0u;
      cp[5] = cw->peak;
      cp[6] = static_cast<unsigned long long>(s);
      cp[7] = (used_bitmap ? kTierBitmap : 0u) | (cw->spilled ? kTierPool : 0u) | (P.rerun ? kTierRerun : 0u) |
              (used_pool2 ? kTierPool2 : 0u);
    }
    __syncwarp();
  }
}

// Host-side launch / occupancy for one instantiation.
template <class DP, bool L2>
cudaError_t launch_t(const SearchParams& P, const float* inv, int blocks, int wpb, cudaStream_t st) {
  const size_t smem = static_cast<size_t>(wpb) * warp_smem_bytes(P.H, P.R, P.C);
  auto* fn = search_kernel<DP, L2>;
  cudaError_t e = open_smem_limit(reinterpret_cast<const void*>(fn));
  if (e != cudaSuccess) return e;
  fn<<<blocks, 32 * wpb, smem, st>>>(P, inv);
  return cudaGetLastError();
}

template <class DP, bool L2>
int occupancy_t(int wpb, size_t smem) {
  int blocks = 0;
  auto* fn = search_kernel<DP, L2>;
  if (open_smem_limit(reinterpret_cast<const void*>(fn)) != cudaSuccess) return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, fn, 32 * wpb, smem) != cudaSuccess) return 0;
  return blocks;
}

// Dispatch on the padded dimension: fixed layouts for common dims, the
// runtime layout (S slots max) otherwise.  G rows in flight per lane group.
#define HG_SEARCH_DISPATCH(FN, L2, ...)                                               \
  switch (pd) {                                                                      \
    case 16: return FN<sk::ExactDist<0, 1, 1, 8>, L2>(__VA_ARGS__);                                 \
    case 32: return FN<sk::ExactDist<0, 2, 2, 8>, L2>(__VA_ARGS__);                                 \
    case 64: return FN<sk::ExactDist<1, 0, 2, 8>, L2>(__VA_ARGS__);                                 \
    case 96: return FN<sk::ExactDist<1, 2, 4, 4>, L2>(__VA_ARGS__);                                 \
    case 112: return FN<sk::ExactDist<1, 3, 5, 4>, L2>(__VA_ARGS__);                                \
    case 128: return FN<sk::ExactDist<2, 0, 4, 4>, L2>(__VA_ARGS__);                                \
    case 256: return FN<sk::ExactDist<4, 0, 8, 2>, L2>(__VA_ARGS__);                                \
    case 512: return FN<sk::ExactDist<8, 0, 16, 2>, L2>(__VA_ARGS__);                               \
    case 768: return FN<sk::ExactDist<12, 0, 24, 1>, L2>(__VA_ARGS__);                              \
    case 960: return FN<sk::ExactDist<15, 0, 30, 1>, L2>(__VA_ARGS__);                              \
    case 1024: return FN<sk::ExactDist<16, 0, 32, 1>, L2>(__VA_ARGS__);                             \
    default: break;                                                                  \
  }                                                                                  \
  {                                                                                  \
    const int S_ = 2 * static_cast<int>(pd / 64) + static_cast<int>((pd % 64) / 16); \
    if (S_ <= 5) return FN<sk::ExactDist<-1, 0, 5, 4>, L2>(__VA_ARGS__);                            \
    if (S_ <= 9) return FN<sk::ExactDist<-1, 0, 9, 2>, L2>(__VA_ARGS__);                            \
    if (S_ <= 17) return FN<sk::ExactDist<-1, 0, 17, 2>, L2>(__VA_ARGS__);                          \
    if (S_ <= 33) return FN<sk::ExactDist<-1, 0, 33, 1>, L2>(__VA_ARGS__);                          \
  }

// The same in the NEON order: chain length pd / 16, rows in pairs.
#define HG_SEARCH_DISPATCH_NEON(FN, L2, ...)                                      \
  switch (pd) {                                                                  \
    case 16: return FN<sk::NeonDist<1, 8>, L2>(__VA_ARGS__);                     \
    case 32: return FN<sk::NeonDist<2, 8>, L2>(__VA_ARGS__);                     \
    case 64: return FN<sk::NeonDist<4, 8>, L2>(__VA_ARGS__);                     \
    case 96: return FN<sk::NeonDist<6, 4>, L2>(__VA_ARGS__);                     \
    case 112: return FN<sk::NeonDist<7, 4>, L2>(__VA_ARGS__);                    \
    case 128: return FN<sk::NeonDist<8, 4>, L2>(__VA_ARGS__);                    \
    case 256: return FN<sk::NeonDist<16, 2>, L2>(__VA_ARGS__);                   \
    case 512: return FN<sk::NeonDist<32, 2>, L2>(__VA_ARGS__);                   \
    case 960: return FN<sk::NeonDist<60, 2, false>, L2>(__VA_ARGS__);            \
    default: break;                                                              \
  }                                                                              \
  {                                                                              \
    const int NC_ = static_cast<int>(pd / 16);                                   \
    if (NC_ <= 8) return FN<sk::NeonDist<-8, 4>, L2>(__VA_ARGS__);               \
    if (NC_ <= 16) return FN<sk::NeonDist<-16, 2>, L2>(__VA_ARGS__);             \
    if (NC_ <= 32) return FN<sk::NeonDist<-32, 2>, L2>(__VA_ARGS__);             \
    if (NC_ <= 66) return FN<sk::NeonDist<-66, 2, false>, L2>(__VA_ARGS__);      \
  }

// compressed-precision traversal layouts per padded width (rows of pdc
// elements); ORD is the summation order of the exact rerank
#define HG_SEARCH_APPROX_DISPATCH(FN, PREC, L2, ORD, ...)                       \
  switch (pdc) {                                                                 \
    case 128: return FN<sk::ApproxDist<4, 16, PREC, ORD>, L2>(__VA_ARGS__);     \
    case 256: return FN<sk::ApproxDist<4, 32, PREC, ORD>, L2>(__VA_ARGS__);     \
    case 512: return FN<sk::ApproxDist<2, 32, PREC, ORD>, L2>(__VA_ARGS__);     \
    case 1024: return FN<sk::ApproxDist<1, 32, PREC, ORD>, L2>(__VA_ARGS__);    \
    default: break;                                                              \
  }

}  // namespace sk
}  // namespace hg
