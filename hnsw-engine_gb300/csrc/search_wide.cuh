// search_wide.cuh -- several warps per query, for the compressed-precision
// forms (FP16 / FP8 rows + exact FP32 rerank), where recall rather than the
// reference's visit order is the bar.
//
// One CTA of kWW warps walks one query.  The descent over the upper layers is
// the one-warp kernel's (warp 0).  Layer 0 is a beam search: the beam holds
// the ef best keys seen, sorted; each step the warps expand the kWW best
// entries not yet expanded (one neighbour list each, distances on compressed
// rows, a visited hash shared by the CTA), warp 0 merges the new keys into the
// beam, and the walk ends when every beam entry has been expanded.  A step
// costs about one expansion of the one-warp kernel, so a query needs about
// 1/kWW of the sequential steps.  The beam's eligible entries then take the
// same exact FP32 rerank and output as the one-warp kernel.  A query whose
// visited set outgrows the hash goes to the overflow list (the rerun pass).
#pragma once

#include "search_kernel.cuh"

namespace hg {
namespace sk {

constexpr int kWW = 4;                    // warps per query
constexpr uint32_t kWideHashLog = 13;     // shared visited hash: 8,192 epoch-tagged ids
constexpr uint32_t kWideHash = 1u << kWideHashLog;
constexpr uint32_t kWideHashLimit = kWideHash / 8 * 5;  // inserts before the query overflows
constexpr uint32_t kWideSteps = 1u << 16;               // bound of the layer-0 loop

// control words after the stage: item, selected count, beam length, visited
// count, overflow, the scan hint (every beam entry before it is expanded),
// then the selected ids
enum : int { kCtlItem = 0, kCtlNsel = 1, kCtlLen = 2, kCtlVisits = 3, kCtlOvf = 4, kCtlHint = 5, kCtlSel = 8, kCtlWords = 16 };

__host__ __device__ inline uint32_t wide_smem_bytes(uint32_t R) {
  return 4u * kWideHash + 8u * R + 8u * 32u * kWW + 4u * kCtlWords;
}

// beam keys: (distance bits << 32) | (id << 1) | expanded; setting the flag
// keeps the (distance, id) order
__device__ __forceinline__ uint64_t wkey(float d, uint32_t id) { return mkkey(d, id << 1); }
__device__ __forceinline__ uint32_t wkey_id(uint64_t k) { return static_cast<uint32_t>(k) >> 1; }

// Insert tag | id into the CTA's hash; true if it was not there.  Ids are
// below 2^24 (tagged mode).  A probe run past the table marks an overflow.
__device__ __forceinline__ bool wide_visit(uint32_t* hash, uint32_t id, uint32_t tag, uint32_t* ovf) {
  const uint32_t key = tag | id;
  uint32_t p = (id * 0x9E3779B1u) >> (32 - kWideHashLog);
  for (uint32_t t = 0; t < kWideHash; ++t) {
    const uint32_t v = *reinterpret_cast<volatile const uint32_t*>(&hash[p]);
    if ((v & 0xFF000000u) != tag) {  // a slot of an earlier query: free
      const uint32_t old = atomicCAS(&hash[p], v, key);
      if (old == v) return true;
      if (old == key) return false;
      continue;  // taken meanwhile by another id: look at the slot again
    }
    if (v == key) return false;
    p = (p + 1) & (kWideHash - 1u);
  }
  *ovf = 1u;
  return false;
}

template <class DP, bool L2>
__global__ void __launch_bounds__(32 * kWW) wide_kernel(SearchParams P, const float* __restrict__ inv_norm) {
  extern __shared__ __align__(16) unsigned char smem[];
  uint32_t* hash = reinterpret_cast<uint32_t*>(smem);
  uint64_t* beam = reinterpret_cast<uint64_t*>(smem + 4u * kWideHash);
  uint64_t* stage = beam + P.R;  // kWW x 32 keys
  uint32_t* ctl = reinterpret_cast<uint32_t*>(stage + 32 * kWW);
  const int lane = threadIdx.x & 31;
  const uint32_t warp = threadIdx.x >> 5;
  for (uint32_t i = threadIdx.x; i < kWideHash; i += blockDim.x) hash[i] = 0u;  // epoch 0: every slot free
  __syncthreads();

  DP dp;
  dp.init(P);
  uint32_t nq = P.nq_dev ? min(*P.nq_dev, P.nq) : P.nq;
  if (P.lpt_sizes) {
    nq = 0;
    for (uint32_t b = 0; b < P.lpt_buckets; ++b) nq += P.lpt_sizes[b];
    nq = min(nq, P.nq);
  }
  uint32_t epoch = 0;

  for (;;) {
    if (threadIdx.x == 0) ctl[kCtlItem] = atomicAdd(P.work, 1u);
    __syncthreads();
    const uint32_t item = ctl[kCtlItem];
    if (item >= nq) break;
    uint32_t q;
    if (P.lpt_sizes) {  // largest-ef bucket first
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
    uint32_t k = P.kq ? P.kq[q] : P.k_all;
    uint32_t ef = P.efq ? P.efq[q] : P.ef_all;
    if (ef == 0) ef = P.ef_default;
    if (ef < k) ef = k;
    const bool refuse = q < P.nq && (ef > P.R || k > P.k_stride || k == 0);
    if (refuse && threadIdx.x == 0) atomicExch(P.err, 1u);
    if (q >= P.nq || refuse) {  // (empty graphs never come here: the one-warp kernel pads them)
      __syncthreads();
      continue;
    }
    if (++epoch == 256u) {  // 8-bit epochs: clear the hash every 255 queries
      for (uint32_t i = threadIdx.x; i < kWideHash; i += blockDim.x) hash[i] = 0u;
      __syncthreads();
      epoch = 1;
    }
    const uint32_t tag = epoch << 24;
    dp.load_query(P, P.queries + static_cast<size_t>(q) * P.dim, inv_norm, q, lane);

    // ---- entry point + greedy descent (search_layer.cpp:29-56), warp 0 ----
    if (warp == 0) {
      uint32_t cur = P.entry;
      float cur_d = dp.template dists<L2>(P, cur, 1u, lane);
      cur_d = __shfl_sync(kFull, cur_d, 0);
      for (int lc = P.max_level; lc > 0; --lc) {
        bool changed = true;
        while (changed) {
          changed = false;
          const uint32_t* lst = P.up + static_cast<size_t>(__ldg(P.up_blk + cur) + (lc - 1)) * P.up_stride;
          for (uint32_t c0 = 0; c0 < P.M; c0 += 32) {
            const uint32_t j = c0 + lane;
            const uint32_t id = j < P.M ? __ldg(lst + j) : kNoId;
            const uint32_t vm = __ballot_sync(kFull, id != kNoId);
            if (!vm) break;
            const float d = dp.template dists<L2>(P, id, vm, lane);
            const float m = warp_minf(id != kNoId ? d : __int_as_float(0x7f800000));
            if (m < cur_d) {
              const uint32_t hit = __ballot_sync(kFull, id != kNoId && d == m);
              cur = __shfl_sync(kFull, id, __ffs(hit) - 1);
              cur_d = m;
              changed = true;
            }
          }
        }
      }
      if (lane == 0) {
        beam[0] = wkey(cur_d, cur);
        ctl[kCtlLen] = 1u;
        ctl[kCtlVisits] = 1u;
        ctl[kCtlOvf] = 0u;
        ctl[kCtlHint] = 0u;
        uint32_t dummy = 0;
        wide_visit(hash, cur, tag, &dummy);
      }
    }
    __syncthreads();

    // ---- layer 0: beam search, kWW expansions per step ----
    for (uint32_t step = 0;; ++step) {
      if (warp == 0) {  // the best kWW entries not yet expanded, marked as expanded
        const uint32_t len = ctl[kCtlLen];
        uint32_t nsel = 0, next = ctl[kCtlHint];
        for (uint32_t base = next & ~31u; base < len && nsel < kWW; base += 32) {
          const uint32_t i = base + lane;
          const uint64_t v = i < len ? beam[i] : 1ull;
          uint32_t b = __ballot_sync(kFull, i < len && !(v & 1ull));
          while (b && nsel < kWW) {
            const int l = __ffs(b) - 1;
            b &= b - 1;
            if (lane == l) {
              beam[i] = v | 1ull;
              ctl[kCtlSel + nsel] = wkey_id(v);
            }
            next = base + static_cast<uint32_t>(l) + 1u;  // entries before it are all expanded now
            ++nsel;
          }
        }
        __syncwarp();
        if (lane == 0) {
          ctl[kCtlNsel] = (ctl[kCtlOvf] || step >= kWideSteps) ? 0u : nsel;
          ctl[kCtlHint] = next;
        }
      }
      __syncthreads();
      const uint32_t nsel = ctl[kCtlNsel];
      if (nsel == 0) break;
      // expand: warp w takes the w-th selected entry
      uint64_t key = kMaxKey;
      if (warp < nsel) {
        const uint32_t cid = ctl[kCtlSel + warp];
        const uint32_t* lst = P.l0 + static_cast<size_t>(cid) * P.l0_stride;
        const uint32_t id = static_cast<uint32_t>(lane) < P.M0 ? __ldg(lst + lane) : kNoId;  // M0 <= 32
        const bool valid = id != kNoId;
        const uint32_t vm = __ballot_sync(kFull, valid);
        bool first = valid;
        if (P.dedup && valid) first = (__ffs(__match_any_sync(vm, id)) - 1) == lane;
        bool fresh = false;
        if (first) fresh = wide_visit(hash, id, tag, &ctl[kCtlOvf]);
        const uint32_t U = __ballot_sync(kFull, fresh);
        if (U) {
          if (lane == 0) atomicAdd(&ctl[kCtlVisits], static_cast<uint32_t>(__popc(U)));
          const float d = dp.template dists<L2>(P, id, U, lane);
          if (fresh) key = wkey(d, id);
        }
      }
      stage[warp * 32 + lane] = key;
      __syncthreads();
      // merge (warp 0): the new keys of all expanded lists are packed to the
      // front of the stage, then sorted and merged into the beam (capacity
      // ef) 32 at a time; a step usually brings fewer than 32
      if (warp == 0) {
        uint32_t len = ctl[kCtlLen];
        const uint64_t worst = len >= ef ? beam[ef - 1] : kMaxKey;
        uint32_t total = 0;
        for (uint32_t w2 = 0; w2 < nsel; ++w2) {
          const uint64_t v = stage[w2 * 32 + lane];
          const bool keep = v != kMaxKey && v < worst;  // no better than the worst kept: dropped
          const uint32_t b = __ballot_sync(kFull, keep);
          __syncwarp();
          if (keep) stage[total + __popc(b & ((1u << lane) - 1u))] = v;  // never past what was read
          total += __popc(b);
          __syncwarp();
        }
        uint32_t hint = ctl[kCtlHint];
        for (uint32_t base = 0; base < total; base += 32) {
          const int m = static_cast<int>(min(32u, total - base));
          uint64_t v = lane < m ? stage[base + lane] : kMaxKey;
          v = warp_sort32(v, lane);
          __syncwarp();
          stage[base + lane] = v;  // base + 32 <= 32 * kWW
          __syncwarp();
          // the smallest new key lands at its rank: the hint may not pass it
          hint = min(hint, static_cast<uint32_t>(lower_bound(beam, static_cast<int>(len), stage[base])));
          len = static_cast<uint32_t>(warp_merge(beam, static_cast<int>(len), static_cast<int>(ef),
                                                 stage + base, m, lane));
        }
        if (lane == 0) ctl[kCtlHint] = hint;
        if (lane == 0) {
          ctl[kCtlLen] = len;
          if (ctl[kCtlVisits] > kWideHashLimit) ctl[kCtlOvf] = 1u;
        }
      }
      __syncthreads();
    }

    if (ctl[kCtlOvf]) {  // the visited set outgrew the hash: the rerun pass answers this query
      if (threadIdx.x == 0) {
        const uint32_t o = atomicAdd(P.ovf_count, 1u);
        if (o < P.nq) P.ovf_list[o] = q;  // at most one entry per query of the batch
      }
      __syncthreads();
      continue;
    }
    // ---- the beam's eligible entries, in beam order, take the exact rerank and the output ----
    if (warp == 0) {
      const int s = static_cast<int>(min(ctl[kCtlLen], ef));
      const uint32_t* fb = nullptr;
      if (P.fsel) {
        const int32_t f = P.fsel[q];
        if (f >= 0) fb = P.fbits[f];
      }
      const bool filtered = fb != nullptr || P.deleted_any != 0;
      uint32_t* prow = P.pool_out + static_cast<size_t>(q) * P.pool_stride;
      int n = 0;
      for (int base = 0; base < s; base += 32) {
        const int i = base + lane;
        const uint32_t id = i < s ? wkey_id(beam[i]) : 0u;
        const bool ok = i < s && (!filtered || (bit_of(P.alive, id) && (!fb || bit_of(fb, id))));
        const uint32_t b = __ballot_sync(kFull, ok);
        if (ok) prow[n + __popc(b & ((1u << lane) - 1u))] = id;
        n += __popc(b);
      }
      if (P.rerank_factor) {
        const uint64_t depth = max(32ull, static_cast<unsigned long long>(P.rerank_factor) * k);
        if (static_cast<uint64_t>(n) > depth) n = static_cast<int>(depth);
      }
      if (lane == 0) P.pool_n[q] = static_cast<uint32_t>(n);
      __syncwarp();
      fused_rerank<typename DP::Exact, L2>(P.vecs, P.pd, P.dim, P.queries + static_cast<size_t>(q) * P.dim,
                                          inv_norm ? inv_norm[q] : 1.0f, inv_norm != nullptr, prow, n, beam, stage,
                                          static_cast<int>(P.R), lane);
      const int m = n < static_cast<int>(k) ? n : static_cast<int>(k);
      QueryOut* row = static_cast<QueryOut*>(P.out) + static_cast<size_t>(q) * P.k_stride;
      for (uint32_t j = lane; j < P.k_stride; j += 32) {
        QueryOut o;
        if (static_cast<int>(j) < m) {
          const uint64_t kk = beam[j];
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
      if (P.done) signal_done(P.done, q, lane);
    }
    __syncthreads();
  }
}

template <class DP, bool L2>
cudaError_t wide_launch_t(const SearchParams& P, const float* inv, int blocks, cudaStream_t st) {
  auto* fn = wide_kernel<DP, L2>;
  cudaError_t e = open_smem_limit(reinterpret_cast<const void*>(fn));
  if (e != cudaSuccess) return e;
  fn<<<blocks, 32 * kWW, wide_smem_bytes(P.R), st>>>(P, inv);
  return cudaGetLastError();
}

template <class DP, bool L2>
int wide_occupancy_t(size_t smem) {
  int blocks = 0;
  auto* fn = wide_kernel<DP, L2>;
  if (open_smem_limit(reinterpret_cast<const void*>(fn)) != cudaSuccess) return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, fn, 32 * kWW, smem) != cudaSuccess) return 0;
  return blocks;
}

}  // namespace sk
}  // namespace hg
