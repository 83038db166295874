// build_graph.cu -- graph construction on the GPU: the linking half of
// Index::add_batch (reference src/index.cpp:145-306), for nodes whose
// vectors, levels and upper blocks the host has already stored in the
// reference's layout (its sequential half, src/index.cpp:101-121, run by the
// host builder's store step, so levels are the reference's draws).
//
// The reference links nodes one at a time (or a few at a time on threads):
// each insertion descends the upper layers greedily, runs Alg. 2 with
// ef_construction on each of its layers, keeps M neighbours by Alg. 4 and
// adds the reverse edges, re-choosing a full list by Alg. 4.  Here the new
// nodes are linked in waves.  A wave [a, b) is linked against the graph of
// nodes [0, a):
//   1. insert_kernel, one warp per new node: the greedy descent, then per
//      layer a beam search of width ef_construction (the beam is Alg. 2's
//      result set; an entry is expanded once; the walk ends when every entry
//      is expanded, which is when Alg. 2's closest candidate lies beyond the
//      worst result), then Alg. 4 over the beam.  The node's own list is
//      written, and each chosen neighbour gets a proposal (distance, new
//      node) in its inbox for that layer.  The beam of a layer is the entry
//      set of the next one, as in the reference.
//   2. link_kernel, one warp per (node, layer) with proposals: the list and
//      the proposals are merged; if they fit the degree cap the proposals are
//      appended (closest first), else the union is re-chosen by Alg. 4, as
//      the reference does for each reverse edge of a full list.
// New nodes of one wave do not see each other during their searches (they
// are linked to each other through later waves' reverse edges and lists),
// so waves are kept a small fraction of the graph they join: the first
// nodes are linked one per wave, later waves grow with the graph.  With
// peer linking (optional), peer_kernel runs between the two: each new node
// re-chooses its list among its neighbours and the wave's nodes that chose
// the same neighbours, which lets waves be larger.  The graph differs from a
// sequential build, as a threaded reference build does; it is judged on
// recall.
//
// Distances are FP32, eight lanes per row (16-byte loads, a three-step
// shuffle reduction); the order of the sum is not the reference's (the
// graph is not meant to be bit-identical).  Visited sets are the beam
// walk's forgetful epoch-tagged hash (ids below 2^24).  Every loop is
// bounded; a wave that exceeds a bound raises the error word and the call
// fails.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

#include "hnswgpu_device.h"
#include "search_beam.cuh"

namespace hg {
namespace gbuild {

using sk::kFull;
using sk::kMaxKey;

constexpr int kWarps = 4;              // warps per block
constexpr int kE = 2;                  // lists expanded per beam step
constexpr int kChunks = 2;             // a list holds up to 64 ids: two warp-wide chunks
constexpr int kMaxDegree = 64;         // M0 = 2M <= 64
constexpr uint32_t kSteps = 1u << 16;  // bound of one layer's beam loop
constexpr uint32_t kInboxCap = 64;     // proposals kept per (node, layer) and wave
constexpr int kFresh = 32 * kE * kChunks;

enum : uint32_t { kErrSteps = 1u };

struct BuildParams {
  const float* vecs;        // count x pd, prepared rows
  uint32_t* l0;             // count x l0_stride: [n, ids...]
  uint32_t* up;             // upper blocks of up_stride words: [n, ids...]
  const uint32_t* up_blk;   // per node with level >= 1: block index of its level 1
  const uint8_t* levels;    // count
  const uint32_t* blk_node; // per upper block: its node
  const uint8_t* blk_level; // per upper block: its level
  uint32_t count, pd, M, M0, efc, l0_stride, up_stride;
  uint32_t H, R;            // visited-hash slots per warp, beam capacity (>= efc, multiple of 32)
  int32_t l2;               // 1: squared L2, 0: 1 - dot (inner product, cosine on unit rows)
  uint32_t* inbox_n;        // per slot: proposals received this wave
  uint64_t* inbox;          // per slot: kInboxCap keys (distance, new node)
  uint32_t* touched;        // slots with proposals this wave
  uint32_t* touched_n;
  unsigned long long* dropped;  // proposals beyond an inbox's capacity (diagnostic)
  uint32_t* err;
};

// slot of (node, layer): layer 0 -> node; layer l >= 1 -> count + block
__device__ __forceinline__ uint32_t slot_of(const BuildParams& P, uint32_t node, int lc) {
  return lc == 0 ? node : P.count + __ldg(P.up_blk + node) + static_cast<uint32_t>(lc - 1);
}
__device__ __forceinline__ uint32_t* list_of(const BuildParams& P, uint32_t node, int lc) {
  return lc == 0 ? P.l0 + static_cast<size_t>(node) * P.l0_stride
                 : P.up + static_cast<size_t>(__ldg(P.up_blk + node) + static_cast<uint32_t>(lc - 1)) * P.up_stride;
}

__host__ __device__ inline uint32_t insert_warp_bytes(uint32_t pd, uint32_t H, uint32_t R) {
  // query row | hash | beam A, B | stage keys | fresh ids | fresh distances | kept ids, distances
  return 4u * pd + 4u * H + 16u * R + 8u * kFresh + 4u * kFresh + 4u * kFresh + 8u * kMaxDegree;
}
__host__ __device__ inline uint32_t link_warp_bytes(uint32_t pd) {
  // row | keys (list + inbox) | two merge buffers | ids | distances | kept ids, distances
  return 4u * pd + 24u * (kMaxDegree + kInboxCap) + 8u * kMaxDegree + 8u * kMaxDegree;
}

// Distances from the row in shared memory qs to rows ids[0..n) into out:
// eight lanes per row, four rows per pass, two passes in flight.
template <bool L2>
__device__ __forceinline__ void row_dists(const BuildParams& P, const float* qs, const uint32_t* ids, int n,
                                          float* out, int lane) {
  const int sub = lane & 7, grp = lane >> 3;
  const uint32_t nv = P.pd >> 2;
  const float4* q4 = reinterpret_cast<const float4*>(qs);
  for (int base = 0; base < n; base += 8) {
    float acc[2] = {0.0f, 0.0f};
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int r = base + 4 * h + grp;
      if (r < n) {
        const float4* row = reinterpret_cast<const float4*>(P.vecs + static_cast<size_t>(ids[r]) * P.pd);
#pragma unroll 4
        for (uint32_t f = sub; f < nv; f += 8) {
          const float4 x = __ldg(row + f);
          const float4 y = q4[f];
          if (L2) {
            const float d0 = x.x - y.x, d1 = x.y - y.y, d2 = x.z - y.z, d3 = x.w - y.w;
            acc[h] = __fmaf_rn(d0, d0, acc[h]);
            acc[h] = __fmaf_rn(d1, d1, acc[h]);
            acc[h] = __fmaf_rn(d2, d2, acc[h]);
            acc[h] = __fmaf_rn(d3, d3, acc[h]);
          } else {
            acc[h] = __fmaf_rn(x.x, y.x, acc[h]);
            acc[h] = __fmaf_rn(x.y, y.y, acc[h]);
            acc[h] = __fmaf_rn(x.z, y.z, acc[h]);
            acc[h] = __fmaf_rn(x.w, y.w, acc[h]);
          }
        }
      }
    }
#pragma unroll
    for (int h = 0; h < 2; ++h) {
#pragma unroll
      for (int o = 1; o < 8; o <<= 1) acc[h] += __shfl_xor_sync(kFull, acc[h], o);
      const int r = base + 4 * h + grp;
      if (sub == 0 && r < n) out[r] = L2 ? acc[h] : 1.0f - acc[h];
    }
  }
  __syncwarp();
}

// Distance between rows a and b, computed by the eight lanes of a group (the
// whole warp calls it in uniform control flow; every lane gets its group's).
template <bool L2>
__device__ __forceinline__ float pair_dist(const BuildParams& P, uint32_t a, uint32_t b, int sub) {
  const uint32_t nv = P.pd >> 2;
  const float4* ra = reinterpret_cast<const float4*>(P.vecs + static_cast<size_t>(a) * P.pd);
  const float4* rb = reinterpret_cast<const float4*>(P.vecs + static_cast<size_t>(b) * P.pd);
  float acc = 0.0f;
#pragma unroll 4
  for (uint32_t f = sub; f < nv; f += 8) {
    const float4 x = __ldg(ra + f);
    const float4 y = __ldg(rb + f);
    if (L2) {
      const float d0 = x.x - y.x, d1 = x.y - y.y, d2 = x.z - y.z, d3 = x.w - y.w;
      acc = __fmaf_rn(d0, d0, acc);
      acc = __fmaf_rn(d1, d1, acc);
      acc = __fmaf_rn(d2, d2, acc);
      acc = __fmaf_rn(d3, d3, acc);
    } else {
      acc = __fmaf_rn(x.x, y.x, acc);
      acc = __fmaf_rn(x.y, y.y, acc);
      acc = __fmaf_rn(x.z, y.z, acc);
      acc = __fmaf_rn(x.w, y.w, acc);
    }
  }
#pragma unroll
  for (int o = 1; o < 8; o <<= 1) acc += __shfl_xor_sync(kFull, acc, o);
  return L2 ? acc : 1.0f - acc;
}

// Alg. 4 (src/index.cpp:127-141): walk the candidates cand[0..nc) in
// (distance, id) order and keep one unless a kept neighbour is strictly
// closer to it than the base node is, until m are kept.  Keys carry the id
// shifted left by SH.  Four candidates are tested per round, one per
// eight-lane group, against every kept neighbour and each other; the
// decisions are then taken in order.  Returns the number kept (kid / kd).
template <bool L2, int SH>
__device__ int select_neighbours(const BuildParams& P, const uint64_t* cand, int nc, int m, uint32_t* kid, float* kd,
                                 int lane) {
  const int sub = lane & 7, grp = lane >> 3;
  int nk = 0;
  for (int i0 = 0; i0 < nc && nk < m; i0 += 4) {
    const int ci = i0 + grp;
    const bool have = ci < nc;
    const uint64_t key = have ? cand[ci] : cand[i0];
    const uint32_t cid = static_cast<uint32_t>(key) >> SH;
    const float cd = sk::key_dist(key);
    bool dom = !have;
    for (int j = 0; j < nk; ++j) {
      if (__all_sync(kFull, dom)) break;
      const float d = pair_dist<L2>(P, cid, kid[j], sub);
      dom = dom || d < cd;
    }
    // distances to the earlier candidates of this round (used if kept)
    float dpre[3];
#pragma unroll
    for (int h = 0; h < 3; ++h) {
      const uint32_t other = __shfl_sync(kFull, cid, 8 * h);
      dpre[h] = pair_dist<L2>(P, cid, other, sub);
    }
    // decisions in order (every lane computes them alike)
    bool kept_round[4] = {false, false, false, false};
#pragma unroll
    for (int g = 0; g < 4; ++g) {
      const bool gh = __shfl_sync(kFull, have ? 1 : 0, 8 * g) != 0;
      if (!gh || nk >= m) continue;
      bool gd = __shfl_sync(kFull, dom ? 1 : 0, 8 * g) != 0;
      const float gcd = __shfl_sync(kFull, cd, 8 * g);
#pragma unroll
      for (int h = 0; h < 3; ++h) {
        const float dgh = __shfl_sync(kFull, dpre[h], 8 * g);
        if (h < g && kept_round[h] && dgh < gcd) gd = true;
      }
      if (!gd) {
        const uint32_t gid = __shfl_sync(kFull, cid, 8 * g);
        if (lane == 0) {
          kid[nk] = gid;
          kd[nk] = gcd;
        }
        kept_round[g] = true;
        ++nk;
      }
    }
    __syncwarp();
  }
  return nk;
}

// Sort n <= 128 unique keys of a[] ascending: each 32-key chunk is sorted in
// place, then the chunks are merged one by one through the ping-pong pair
// t0 / t1 (128 keys each, apart from a).  Returns the buffer holding the result.
__device__ uint64_t* sort_small(uint64_t* a, uint64_t* t0, uint64_t* t1, int n, int lane) {
  for (int base = 0; base < n; base += 32) {
    const int c = min(32, n - base);
    uint64_t v = lane < c ? a[base + lane] : kMaxKey;
    v = sk::warp_sort32(v, lane);
    __syncwarp();
    if (lane < c) a[base + lane] = v;
  }
  __syncwarp();
  if (n <= 32) return a;
  uint32_t unused = 0xFFFFFFFFu;
  uint64_t* src = a;
  uint64_t* dst = t0;
  int len = 32;
  for (int base = 32; base < n; base += 32) {
    const int c = min(32, n - base);
    len = sk::merge_path(src, len, dst, 128, a + base, c, &unused, lane);
    __syncwarp();
    src = dst;
    dst = dst == t0 ? t1 : t0;
  }
  return src;
}

// ---------------------------------------------------------------------------
// 1. search + select for each node of the wave [a, b)
// ---------------------------------------------------------------------------
template <bool L2>
__global__ void __launch_bounds__(32 * kWarps) insert_kernel(BuildParams P, uint32_t a, uint32_t b, uint32_t entry,
                                                            int top) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const uint32_t node = a + blockIdx.x * kWarps + static_cast<uint32_t>(wib);
  if (node >= b) return;
  unsigned char* base = smem + static_cast<size_t>(wib) * insert_warp_bytes(P.pd, P.H, P.R);
  float* qs = reinterpret_cast<float*>(base);
  uint32_t* hash = reinterpret_cast<uint32_t*>(base + 4u * P.pd);
  uint64_t* beamA = reinterpret_cast<uint64_t*>(hash + P.H);
  uint64_t* beamB = beamA + P.R;
  uint64_t* stage = beamB + P.R;
  uint32_t* fid = reinterpret_cast<uint32_t*>(stage + kFresh);
  float* fdist = reinterpret_cast<float*>(fid + kFresh);
  uint32_t* kid = reinterpret_cast<uint32_t*>(fdist + kFresh);
  float* kd = reinterpret_cast<float*>(kid + kMaxDegree);

  for (uint32_t i = lane; i < P.H; i += 32) hash[i] = 0u;
  {
    const float4* src = reinterpret_cast<const float4*>(P.vecs + static_cast<size_t>(node) * P.pd);
    float4* dst = reinterpret_cast<float4*>(qs);
    for (uint32_t f = lane; f < (P.pd >> 2); f += 32) dst[f] = __ldg(src + f);
  }
  __syncwarp();
  const int level = P.levels[node];

  // entry point and greedy descent above the node's level (Alg. 1, lines 5-7)
  if (lane == 0) fid[0] = entry;
  __syncwarp();
  row_dists<L2>(P, qs, fid, 1, fdist, lane);
  uint32_t cur_id = entry;
  float cur_d = fdist[0];
  for (int lc = top; lc > level; --lc) {
    for (uint32_t guard = 0; guard < P.count; ++guard) {
      const uint32_t* lst = list_of(P, cur_id, lc);
      const uint32_t cnt = min(__ldg(lst), P.M);
      const uint32_t id = static_cast<uint32_t>(lane) < cnt ? __ldg(lst + 1 + lane) : kNoId;
      __syncwarp();
      if (id != kNoId) fid[lane] = id;
      __syncwarp();
      row_dists<L2>(P, qs, fid, static_cast<int>(cnt), fdist, lane);
      const float d = id != kNoId ? fdist[lane] : __int_as_float(0x7f800000);
      const float mn = sk::warp_minf(d);
      if (!(mn < cur_d)) break;
      const uint32_t hit = __ballot_sync(kFull, id != kNoId && d == mn);
      cur_id = __shfl_sync(kFull, id, __ffs(hit) - 1);
      cur_d = mn;
      __syncwarp();
    }
  }

  // layers min(level, top) .. 0: beam search, Alg. 4, own list, proposals
  uint64_t* cur = beamA;
  uint64_t* oth = beamB;
  if (lane == 0) cur[0] = sk::wkey(cur_d, cur_id);
  int blen = 1;
  __syncwarp();
  const int efc = static_cast<int>(P.efc);
  const uint32_t hlimit = P.H / 8u * 5u;
  uint32_t epoch = 0;
  for (int lc = min(level, top); lc >= 0; --lc) {
    const uint32_t cap = lc == 0 ? P.M0 : P.M;
    if (++epoch == 256u) {
      for (uint32_t i = lane; i < P.H; i += 32) hash[i] = 0u;
      __syncwarp();
      epoch = 1;
    }
    sk::BeamVisited V{epoch << 24, 0u, 0u, P.H};
    // the previous layer's beam is this layer's entry set, none expanded yet
    for (int i = lane; i < blen; i += 32) {
      cur[i] &= ~1ull;
      sk::beam_visit(hash, V, sk::wkey_id(cur[i]));
    }
    V.count = static_cast<uint32_t>(blen);
    __syncwarp();
    uint32_t hint = 0;
    bool done = false;
    for (uint32_t step = 0; step < kSteps; ++step) {
      const uint64_t worst = blen >= efc ? (cur[efc - 1] | 1ull) : kMaxKey;
      // the kE best unexpanded entries
      uint32_t selv = kNoId;
      int nsel = 0;
      uint32_t next = hint;
      for (uint32_t b0 = hint & ~31u; b0 < static_cast<uint32_t>(blen) && nsel < kE; b0 += 32) {
        const uint32_t i = b0 + lane;
        const bool live = i < static_cast<uint32_t>(blen);
        const uint64_t v = live ? cur[i] : kMaxKey;
        uint32_t bal = __ballot_sync(kFull, live && !(v & 1ull));
        const uint32_t myid = sk::wkey_id(v);
        while (bal && nsel < kE) {
          const int l = __ffs(bal) - 1;
          bal &= bal - 1;
          if (lane == l) cur[i] = v | 1ull;
          const uint32_t sid = __shfl_sync(kFull, myid, l);
          if (lane == nsel) selv = sid;
          ++nsel;
          next = b0 + static_cast<uint32_t>(l) + 1u;
        }
      }
      hint = next;
      if (nsel == 0) {
        done = true;
        break;
      }
      __syncwarp();
      // the selected lists, then the visited test; fresh ids packed into fid
      int nf = 0;
#pragma unroll
      for (int e = 0; e < kE; ++e) {
        const uint32_t se = __shfl_sync(kFull, selv, e);
        if (e >= nsel) break;
        const uint32_t* lst = list_of(P, se, lc);
        const uint32_t cnt = min(__ldg(lst), cap);
#pragma unroll
        for (int c = 0; c < kChunks; ++c) {
          const uint32_t j = static_cast<uint32_t>(lane + 32 * c);
          const uint32_t id = j < cnt ? __ldg(lst + 1 + j) : kNoId;
          const bool valid = id != kNoId;
          const uint32_t vm = __ballot_sync(kFull, valid);
          if (!vm) break;
          if (V.count + static_cast<uint32_t>(__popc(vm)) > hlimit) {
            // forget: a new epoch holding the beam's ids and this step's fresh ids
            if (++epoch == 256u) {
              for (uint32_t i = lane; i < P.H; i += 32) hash[i] = 0u;
              epoch = 1;
            }
            V.tag = epoch << 24;
            ++V.resets;
            __syncwarp();
            for (int i = lane; i < blen; i += 32) sk::beam_visit(hash, V, sk::wkey_id(cur[i]));
            for (int i = lane; i < nf; i += 32) sk::beam_visit(hash, V, fid[i]);
            V.count = static_cast<uint32_t>(blen + nf);
            __syncwarp();
          }
          const bool fresh = valid && sk::beam_visit(hash, V, id);
          __syncwarp();
          const uint32_t fm = __ballot_sync(kFull, fresh);
          if (fresh) fid[nf + __popc(fm & ((1u << lane) - 1u))] = id;
          nf += __popc(fm);
          V.count += __popc(fm);
        }
      }
      __syncwarp();
      if (nf == 0) continue;
      row_dists<L2>(P, qs, fid, nf, fdist, lane);
      // keys better than the worst kept enter the beam
      int m = 0;
      for (int b0 = 0; b0 < nf; b0 += 32) {
        const int i = b0 + lane;
        uint64_t v = kMaxKey;
        bool keep = false;
        if (i < nf) {
          v = sk::wkey(fdist[i], fid[i]);
          keep = v < worst;
        }
        const uint32_t bal = __ballot_sync(kFull, keep);
        if (keep) stage[m + __popc(bal & ((1u << lane) - 1u))] = v;
        m += __popc(bal);
      }
      __syncwarp();
      blen = sk::merge_keys(cur, oth, blen, efc, stage, m, &hint, V.resets > 0, lane);
    }
    if (!done) {
      if (lane == 0) atomicOr(P.err, kErrSteps);
      return;
    }
    // Alg. 4 over the beam (sorted by distance, then id), M neighbours
    const int nk = select_neighbours<L2, 1>(P, cur, blen, static_cast<int>(P.M), kid, kd, lane);
    uint32_t* own = list_of(P, node, lc);
    for (int j = lane; j < nk; j += 32) own[1 + j] = kid[j];
    if (lane == 0) own[0] = static_cast<uint32_t>(nk);
    // proposals: the reverse edges (Alg. 1, lines 11-16), merged by link_kernel
    for (int j = lane; j < nk; j += 32) {
      const uint32_t t = kid[j];
      const uint32_t s = slot_of(P, t, lc);
      const uint32_t pos = atomicAdd(P.inbox_n + s, 1u);
      if (pos == 0) P.touched[atomicAdd(P.touched_n, 1u)] = s;
      if (pos < kInboxCap) P.inbox[static_cast<size_t>(s) * kInboxCap + pos] = sk::mkkey(kd[j], node);
      else atomicAdd(P.dropped, 1ull);
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------
// 1b. peers: new nodes of the wave that chose the same old neighbours
// ---------------------------------------------------------------------------
// A new node did not see the other new nodes of its wave while it searched.
// The proposals in its chosen neighbours' inboxes name exactly the new nodes
// that chose the same neighbours -- the wave's nodes nearest to it.  Each
// new node re-chooses its own list by Alg. 4 from its neighbours plus those
// peers (up to kPeerCap of them) and proposes itself to the peers it keeps,
// so the reverse-edge merge links the wave's nodes to each other as a
// sequential build would.  This lets waves be larger at the same recall.
constexpr int kPeerCap = 96;  // peers considered per (node, layer); with M <= 32 own ids, 128 keys

__host__ __device__ inline uint32_t peer_warp_bytes(uint32_t pd) {
  // row | keys + two merge buffers (128 each) | ids | distances | kept ids, distances
  return 4u * pd + 24u * 128u + 4u * 128u + 4u * 128u + 8u * kMaxDegree;
}

template <bool L2>
__global__ void __launch_bounds__(32 * kWarps) peer_kernel(BuildParams P, uint32_t a, uint32_t b, int top) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const uint32_t node = a + blockIdx.x * kWarps + static_cast<uint32_t>(wib);
  if (node >= b) return;
  unsigned char* base = smem + static_cast<size_t>(wib) * peer_warp_bytes(P.pd);
  float* row = reinterpret_cast<float*>(base);
  uint64_t* ka = reinterpret_cast<uint64_t*>(base + 4u * P.pd);
  uint64_t* kb = ka + 128;
  uint64_t* kc = kb + 128;
  uint32_t* ids = reinterpret_cast<uint32_t*>(kc + 128);
  float* dist = reinterpret_cast<float*>(ids + 128);
  uint32_t* kid = reinterpret_cast<uint32_t*>(dist + 128);
  float* kd = reinterpret_cast<float*>(kid + kMaxDegree);
  {
    const float4* src = reinterpret_cast<const float4*>(P.vecs + static_cast<size_t>(node) * P.pd);
    float4* dst = reinterpret_cast<float4*>(row);
    for (uint32_t f = lane; f < (P.pd >> 2); f += 32) dst[f] = __ldg(src + f);
  }
  __syncwarp();
  const int level = P.levels[node];
  for (int lc = min(level, top); lc >= 0; --lc) {
    uint32_t* own = list_of(P, node, lc);
    const int nk = static_cast<int>(min(own[0], P.M));
    // the peers: every proposer in the own neighbours' inboxes but this node
    int np = 0;
    for (int j = 0; j < nk && np < kPeerCap; ++j) {
      const uint32_t s = slot_of(P, own[1 + j], lc);
      const int cnt = static_cast<int>(min(P.inbox_n[s], kInboxCap));
      for (int t0 = 0; t0 < cnt && np < kPeerCap; t0 += 32) {
        const int t = t0 + lane;
        uint32_t pid = kNoId;
        if (t < cnt) pid = static_cast<uint32_t>(P.inbox[static_cast<size_t>(s) * kInboxCap + t]);
        const bool take = pid != kNoId && pid != node;
        const uint32_t bal = __ballot_sync(kFull, take);
        const int at = np + __popc(bal & ((1u << lane) - 1u));
        // (peer << 32 | position): unique keys for the sort, peers adjacent
        if (take && at < kPeerCap) ka[at] = (static_cast<uint64_t>(pid) << 32) | static_cast<uint32_t>(at);
        np = min(kPeerCap, np + __popc(bal));
      }
    }
    __syncwarp();
    if (np == 0) continue;
    // unique peers (a peer may have chosen several of the same neighbours)
    const uint64_t* sorted = sort_small(ka, kb, kc, np, lane);
    int nu = 0;
    for (int b0 = 0; b0 < np; b0 += 32) {
      const int i = b0 + lane;
      const bool first = i < np && (i == 0 || (sorted[i] >> 32) != (sorted[i - 1] >> 32));
      const uint32_t bal = __ballot_sync(kFull, first);
      if (first) ids[nu + __popc(bal & ((1u << lane) - 1u))] = static_cast<uint32_t>(sorted[i] >> 32);
      nu += __popc(bal);
    }
    for (int j = lane; j < nk; j += 32) ids[nu + j] = own[1 + j];
    __syncwarp();
    const int nc = nu + nk;
    row_dists<L2>(P, row, ids, nc, dist, lane);
    for (int j = lane; j < nc; j += 32) ka[j] = sk::mkkey(dist[j], ids[j]);
    __syncwarp();
    const uint64_t* cand = sort_small(ka, kb, kc, nc, lane);
    const int nkept = select_neighbours<L2, 0>(P, cand, nc, static_cast<int>(P.M), kid, kd, lane);
    for (int j = lane; j < nkept; j += 32) own[1 + j] = kid[j];
    __syncwarp();
    if (lane == 0) own[0] = static_cast<uint32_t>(nkept);
    // proposals to the kept peers (new nodes of this wave); the old
    // neighbours hold this node's proposal already
    for (int j = lane; j < nkept; j += 32) {
      const uint32_t t = kid[j];
      if (t < a || t >= b) continue;
      const uint32_t sl = slot_of(P, t, lc);
      const uint32_t pos = atomicAdd(P.inbox_n + sl, 1u);
      if (pos == 0) P.touched[atomicAdd(P.touched_n, 1u)] = sl;
      if (pos < kInboxCap) P.inbox[static_cast<size_t>(sl) * kInboxCap + pos] = sk::mkkey(kd[j], node);
      else atomicAdd(P.dropped, 1ull);
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------
// 2. merge the proposals of each touched (node, layer) into its list
// ---------------------------------------------------------------------------
template <bool L2>
__global__ void __launch_bounds__(32 * kWarps) link_kernel(BuildParams P) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  unsigned char* base = smem + static_cast<size_t>(wib) * link_warp_bytes(P.pd);
  float* row = reinterpret_cast<float*>(base);
  uint64_t* ka = reinterpret_cast<uint64_t*>(base + 4u * P.pd);
  uint64_t* kb = ka + (kMaxDegree + kInboxCap);
  uint64_t* kc = kb + (kMaxDegree + kInboxCap);
  uint32_t* ids = reinterpret_cast<uint32_t*>(kc + (kMaxDegree + kInboxCap));
  float* dist = reinterpret_cast<float*>(ids + kMaxDegree);
  uint32_t* kid = reinterpret_cast<uint32_t*>(dist + kMaxDegree);
  float* kd = reinterpret_cast<float*>(kid + kMaxDegree);
  const uint32_t nt = *P.touched_n;
  const uint32_t stride = gridDim.x * kWarps;
  for (uint32_t i = blockIdx.x * kWarps + static_cast<uint32_t>(wib); i < nt; i += stride) {
    const uint32_t s = P.touched[i];
    uint32_t node;
    int lc;
    uint32_t* lst;
    if (s < P.count) {
      node = s;
      lc = 0;
      lst = P.l0 + static_cast<size_t>(node) * P.l0_stride;
    } else {
      const uint32_t blk = s - P.count;
      node = P.blk_node[blk];
      lc = P.blk_level[blk];
      lst = P.up + static_cast<size_t>(blk) * P.up_stride;
    }
    const uint32_t cap = lc == 0 ? P.M0 : P.M;
    const int np = static_cast<int>(min(P.inbox_n[s], kInboxCap));
    const int cnt = static_cast<int>(min(lst[0], cap));
    // the node's current list (ids) and the proposals (keys)
    for (int j = lane; j < cnt; j += 32) ids[j] = lst[1 + j];
    for (int j = lane; j < np; j += 32) ka[j] = P.inbox[static_cast<size_t>(s) * kInboxCap + j];
    __syncwarp();
    // drop proposals already in the list (cannot happen within a wave; kept
    // for robustness)
    int npk = 0;
    for (int b0 = 0; b0 < np; b0 += 32) {
      const int j = b0 + lane;
      bool keep = false;
      uint64_t v = 0;
      if (j < np) {
        v = ka[j];
        const uint32_t src = static_cast<uint32_t>(v);
        keep = true;
        for (int e = 0; e < cnt; ++e) keep = keep && ids[e] != src;
      }
      const uint32_t bal = __ballot_sync(kFull, keep);
      __syncwarp();
      if (keep) ka[npk + __popc(bal & ((1u << lane) - 1u))] = v;
      npk += __popc(bal);
      __syncwarp();
    }
    if (cnt + npk <= static_cast<int>(cap)) {
      // room: the proposals are appended, closest first
      const uint64_t* sorted = sort_small(ka, kb, kc, npk, lane);
      for (int j = lane; j < npk; j += 32) lst[1 + cnt + j] = static_cast<uint32_t>(sorted[j]);
      __syncwarp();
      if (lane == 0) lst[0] = static_cast<uint32_t>(cnt + npk);
    } else {
      // full: Alg. 4 over the old list plus the proposals, cap neighbours
      {
        const float4* src = reinterpret_cast<const float4*>(P.vecs + static_cast<size_t>(node) * P.pd);
        float4* dst = reinterpret_cast<float4*>(row);
        for (uint32_t f = lane; f < (P.pd >> 2); f += 32) dst[f] = __ldg(src + f);
      }
      __syncwarp();
      row_dists<L2>(P, row, ids, cnt, dist, lane);
      for (int j = lane; j < cnt; j += 32) ka[npk + j] = sk::mkkey(dist[j], ids[j]);
      __syncwarp();
      const uint64_t* sorted = sort_small(ka, kb, kc, npk + cnt, lane);
      const int nk = select_neighbours<L2, 0>(P, sorted, npk + cnt, static_cast<int>(cap), kid, kd, lane);
      for (int j = lane; j < nk; j += 32) lst[1 + j] = kid[j];
      __syncwarp();
      if (lane == 0) lst[0] = static_cast<uint32_t>(nk);
    }
    if (lane == 0) P.inbox_n[s] = 0u;
    __syncwarp();
  }
}

}  // namespace gbuild

// ---------------------------------------------------------------------------
// host driver
// ---------------------------------------------------------------------------
namespace {

struct DevMem {
  std::vector<void*> ptrs;
  ~DevMem() {
    for (void* p : ptrs) cudaFree(p);
  }
  template <typename T>
  cudaError_t alloc(T** p, size_t count) {
    void* v = nullptr;
    const cudaError_t e = cudaMalloc(&v, std::max<size_t>(count * sizeof(T), 256));
    if (e == cudaSuccess) ptrs.push_back(v);
    *p = static_cast<T*>(v);
    return e;
  }
};

}  // namespace

int build_graph(hgd_build_args* a, int device, std::string* err) {
  using namespace gbuild;
  auto bad = [&](int code, const std::string& m) {
    *err = "hgd_build_graph: " + m;
    return code;
  };
  if (!a || !a->vectors || !a->level0 || !a->levels || !a->upper_offset) return bad(HGD_EINVAL, "null argument");
  if (a->count >= (1ull << 24)) return bad(HGD_EINVAL, "the GPU builder takes fewer than 2^24 nodes");
  if (a->first > a->count) return bad(HGD_EINVAL, "first exceeds count");
  if (a->M < 2 || 2 * a->M > static_cast<uint64_t>(kMaxDegree)) return bad(HGD_EINVAL, "the GPU builder takes 2 <= M <= 32");
  if (a->padded_dim % 16 != 0 || a->padded_dim == 0 || a->padded_dim > 1024 || a->dim > a->padded_dim)
    return bad(HGD_EINVAL, "padded_dim must be dim rounded up to 16, at most 1024");
  if (a->ef_construction == 0 || a->ef_construction > 1024) return bad(HGD_EINVAL, "ef_construction must be 1..1024");
  a->waves = 0;
  a->dropped_proposals = 0;
  const uint32_t count = static_cast<uint32_t>(a->count);
  const uint32_t first = static_cast<uint32_t>(a->first);
  if (first == count) return HGD_OK;
  const uint32_t M = static_cast<uint32_t>(a->M), M0 = 2 * M;
  const uint32_t pd = static_cast<uint32_t>(a->padded_dim);
  const uint32_t l0_stride = 1 + M0, up_stride = 1 + M;
  const uint32_t efc = static_cast<uint32_t>(std::max<uint64_t>(a->ef_construction, M));

  // upper blocks: node -> first block, block -> (node, level)
  std::vector<uint32_t> up_blk(count, kNoId);
  std::vector<uint32_t> blk_node;
  std::vector<uint8_t> blk_level;
  for (uint32_t i = 0; i < count; ++i) {
    const int L = a->levels[i];
    if (L == 0) continue;
    if (a->upper_offset[i] % up_stride != 0) return bad(HGD_EINVAL, "upper offsets must be whole blocks");
    const uint64_t b0 = a->upper_offset[i] / up_stride;
    if ((b0 + L) * up_stride > a->upper_words) return bad(HGD_EINVAL, "upper offsets exceed the upper array");
    up_blk[i] = static_cast<uint32_t>(b0);
    if (blk_node.size() < b0 + L) {
      blk_node.resize(b0 + L, 0u);
      blk_level.resize(b0 + L, 0u);
    }
    for (int l = 1; l <= L; ++l) {
      blk_node[b0 + l - 1] = i;
      blk_level[b0 + l - 1] = static_cast<uint8_t>(l);
    }
  }
  const uint64_t nblocks = a->upper_words / up_stride;
  blk_node.resize(std::max<uint64_t>(nblocks, 1), 0u);
  blk_level.resize(std::max<uint64_t>(nblocks, 1), 0u);
  const uint64_t slots = count + nblocks;

  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return bad(HGD_ECUDA, cudaGetErrorString(e));
  int sms = 0;
  if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device)) != cudaSuccess)
    return bad(HGD_ECUDA, cudaGetErrorString(e));
  cudaStream_t st = nullptr;
  if ((e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking)) != cudaSuccess)
    return bad(HGD_ECUDA, cudaGetErrorString(e));
  struct StreamGuard {
    cudaStream_t s;
    ~StreamGuard() { cudaStreamDestroy(s); }
  } sg{st};

  DevMem mem;
  BuildParams P{};
  float* d_vecs = nullptr;
  uint32_t *d_l0 = nullptr, *d_up = nullptr, *d_upblk = nullptr, *d_blk_node = nullptr;
  uint8_t *d_levels = nullptr, *d_blk_level = nullptr;
  uint32_t *d_inbox_n = nullptr, *d_touched = nullptr, *d_small = nullptr;
  uint64_t* d_inbox = nullptr;
  unsigned long long* d_dropped = nullptr;
  const uint64_t up_words = std::max<uint64_t>(a->upper_words, 1);
  if (mem.alloc(&d_vecs, static_cast<size_t>(count) * pd) != cudaSuccess ||
      mem.alloc(&d_l0, static_cast<size_t>(count) * l0_stride) != cudaSuccess ||
      mem.alloc(&d_up, up_words) != cudaSuccess || mem.alloc(&d_upblk, count) != cudaSuccess ||
      mem.alloc(&d_levels, count) != cudaSuccess || mem.alloc(&d_blk_node, blk_node.size()) != cudaSuccess ||
      mem.alloc(&d_blk_level, blk_level.size()) != cudaSuccess || mem.alloc(&d_inbox_n, slots) != cudaSuccess ||
      mem.alloc(&d_inbox, slots * kInboxCap) != cudaSuccess || mem.alloc(&d_touched, slots) != cudaSuccess ||
      mem.alloc(&d_small, 4) != cudaSuccess || mem.alloc(&d_dropped, 1) != cudaSuccess)
    return bad(HGD_ENOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(cudaGetLastError()));
  auto up = [&](void* dst, const void* src, size_t bytes) {
    return bytes ? cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, st) : cudaSuccess;
  };
  if ((e = up(d_vecs, a->vectors, static_cast<size_t>(count) * pd * 4)) != cudaSuccess ||
      (e = up(d_l0, a->level0, static_cast<size_t>(count) * l0_stride * 4)) != cudaSuccess ||
      (e = up(d_up, a->upper, a->upper_words * 4)) != cudaSuccess ||
      (e = up(d_upblk, up_blk.data(), static_cast<size_t>(count) * 4)) != cudaSuccess ||
      (e = up(d_levels, a->levels, count)) != cudaSuccess ||
      (e = up(d_blk_node, blk_node.data(), blk_node.size() * 4)) != cudaSuccess ||
      (e = up(d_blk_level, blk_level.data(), blk_level.size())) != cudaSuccess ||
      (e = cudaMemsetAsync(d_inbox_n, 0, slots * 4, st)) != cudaSuccess ||
      (e = cudaMemsetAsync(d_small, 0, 16, st)) != cudaSuccess ||
      (e = cudaMemsetAsync(d_dropped, 0, 8, st)) != cudaSuccess)
    return bad(HGD_ECUDA, std::string("upload: ") + cudaGetErrorString(e));

  P.vecs = d_vecs;
  P.l0 = d_l0;
  P.up = d_up;
  P.up_blk = d_upblk;
  P.levels = d_levels;
  P.blk_node = d_blk_node;
  P.blk_level = d_blk_level;
  P.count = count;
  P.pd = pd;
  P.M = M;
  P.M0 = M0;
  P.efc = efc;
  P.l0_stride = l0_stride;
  P.up_stride = up_stride;
  P.R = (efc + 31u) / 32u * 32u;
  P.H = beam_hash_slots(efc);
  while (P.H / 8u * 5u < 2u * (P.R + static_cast<uint32_t>(kFresh))) P.H <<= 1;
  P.l2 = a->metric == HGD_METRIC_L2 ? 1 : 0;
  P.inbox_n = d_inbox_n;
  P.inbox = d_inbox;
  P.touched = d_touched;
  P.touched_n = d_small;
  P.err = d_small + 1;
  P.dropped = d_dropped;

  const size_t ins_smem = static_cast<size_t>(kWarps) * insert_warp_bytes(pd, P.H, P.R);
  const size_t link_smem = static_cast<size_t>(kWarps) * link_warp_bytes(pd);
  auto* ins = P.l2 ? insert_kernel<true> : insert_kernel<false>;
  auto* lnk = P.l2 ? link_kernel<true> : link_kernel<false>;
  auto* peer = P.l2 ? peer_kernel<true> : peer_kernel<false>;
  const size_t peer_smem = static_cast<size_t>(kWarps) * peer_warp_bytes(pd);
  const bool peers = a->peers != 0;
  if ((e = open_smem_limit(reinterpret_cast<const void*>(ins))) != cudaSuccess ||
      (e = open_smem_limit(reinterpret_cast<const void*>(lnk))) != cudaSuccess ||
      (e = open_smem_limit(reinterpret_cast<const void*>(peer))) != cudaSuccess)
    return bad(HGD_ECUDA, cudaGetErrorString(e));
  int link_blocks = 0;
  if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&link_blocks, lnk, 32 * kWarps, link_smem)) != cudaSuccess)
    return bad(HGD_ECUDA, cudaGetErrorString(e));
  int ins_blocks = 0;
  if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ins_blocks, ins, 32 * kWarps, ins_smem)) != cudaSuccess)
    return bad(HGD_ECUDA, cudaGetErrorString(e));
  if (ins_blocks < 1 || link_blocks < 1) return bad(HGD_EINVAL, "the shared-memory layout does not fit one block");
  link_blocks *= sms;

  // waves: [a, b) joins the graph of nodes [0, a)
  const double frac = a->wave_fraction > 0.0 ? a->wave_fraction : 0.02;
  const uint64_t wmin = a->wave_min ? a->wave_min : 1;
  // largest wave: four (peer linking: sixteen) rounds of the resident warps
  const uint64_t wmax =
      a->wave_max ? a->wave_max : static_cast<uint64_t>(ins_blocks) * sms * kWarps * (a->peers ? 16 : 4);
  uint32_t entry = a->entry_point;
  int top = a->max_level;
  uint32_t at = first;
  if (entry == kNoId) {  // empty graph: the first node is the entry point
    entry = first;
    top = a->levels[first];
    ++at;
  }
  while (at < count) {
    uint64_t w = static_cast<uint64_t>(std::floor(frac * at));
    w = std::min(std::max(w, wmin), wmax);
    const uint32_t b = static_cast<uint32_t>(std::min<uint64_t>(at + w, count));
    const uint32_t blocks = (b - at + kWarps - 1) / kWarps;
    ins<<<blocks, 32 * kWarps, ins_smem, st>>>(P, at, b, entry, top);
    if (peers && b - at > 1) peer<<<blocks, 32 * kWarps, peer_smem, st>>>(P, at, b, top);
    lnk<<<link_blocks, 32 * kWarps, link_smem, st>>>(P);
    if ((e = cudaMemsetAsync(d_small, 0, 4, st)) != cudaSuccess) return bad(HGD_ECUDA, cudaGetErrorString(e));
    if ((e = cudaGetLastError()) != cudaSuccess) return bad(HGD_ECUDA, std::string("launch: ") + cudaGetErrorString(e));
    // the entry point after the wave: the first node that raised the top level
    for (uint32_t i = at; i < b; ++i)
      if (static_cast<int>(a->levels[i]) > top) {
        top = a->levels[i];
        entry = i;
      }
    at = b;
    ++a->waves;
  }
  // the lists come back into staging copies; the caller's arrays change only
  // once every kernel and copy has succeeded
  uint32_t flags[2] = {0, 0};
  unsigned long long dropped = 0;
  std::vector<uint32_t> l0_back(static_cast<size_t>(count) * l0_stride);
  std::vector<uint32_t> up_back(a->upper_words);
  if ((e = cudaMemcpyAsync(flags, d_small, 8, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
      (e = cudaMemcpyAsync(&dropped, d_dropped, 8, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
      (e = cudaMemcpyAsync(l0_back.data(), d_l0, l0_back.size() * 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
      (e = (a->upper_words ? cudaMemcpyAsync(up_back.data(), d_up, a->upper_words * 4, cudaMemcpyDeviceToHost, st)
                           : cudaSuccess)) != cudaSuccess ||
      (e = cudaStreamSynchronize(st)) != cudaSuccess)
    return bad(HGD_ECUDA, std::string("build: ") + cudaGetErrorString(e));
  if (flags[1] & kErrSteps) return bad(HGD_ERUNTIME, "a layer search exceeded its step bound");
  std::copy(l0_back.begin(), l0_back.end(), a->level0);
  std::copy(up_back.begin(), up_back.end(), a->upper);
  a->entry_point = entry;
  a->max_level = top;
  a->dropped_proposals = dropped;
  return HGD_OK;
}

}  // namespace hg
