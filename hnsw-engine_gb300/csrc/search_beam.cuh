// search_beam.cuh -- the throughput walk of the compressed-precision forms:
// one warp per query, several neighbour lists expanded per step, row
// distances on the tensor cores.
//
// The FP16 / FP8 forms are judged on recall (their answers come from an
// exact FP32 rerank), so their walk need not replay the reference's visit
// order.  This kernel walks layer 0 as a beam search: the beam holds the ef
// best keys seen, sorted, each flagged once expanded.  A step
//   1. takes the E best unexpanded beam entries (E = lists_per_step, <= 4),
//   2. loads their neighbour lists together (E independent 128-byte loads),
//   3. tests the ids against the warp's visited set and prefetches the rows
//      of the fresh ones into L2,
//   4. computes the distances of all fresh rows, 16 rows per group, with
//      mma.sync m16n8k16 (rows as A; the query as B, split into a high and a
//      low FP16 part in columns 0 and 1, so the query keeps ~22 bits),
//   5. merges the keys better than the beam's worst into the beam.
// The walk ends when every beam entry is expanded.  The work per expansion
// is a fraction of the one-warp replay kernel's, and the E lists' rows are
// in flight together, so fewer dependent memory round trips lie on the
// query's path.  The work is a gathered matrix-vector product (one query
// column), so the register-operand MMA fits it: its operands come straight
// from the gathered loads, with no shared-memory staging on the path.
//
// Filters and deletes follow Alg. 2's split (the FILT instantiation): every
// accepted key enters the beam (the candidates, capacity a multiple of 32
// from ef), eligible ones also a result list (capacity ef); a key is
// accepted while fewer than ef results exist or it beats the worst result,
// and an entry is expanded only while it does not lie beyond the worst
// result.  The beam is bounded where Alg. 2's candidate queue is not, so
// very restrictive filters lose recall; the batch call routes those to the
// exact scan (filter_scan_permille).
//
// Distances.  The compressed rows hold x' (FP16, or E4M3 with a per-row
// scale s: x = s x'); per row the copy also stores n = s^2 |x'|^2.  With the
// query's dot product d = q . x' from the tensor cores:
//     L2:  |q|^2 - 2 s d + n        IP / cosine:  1 - s d
// These are the rows the CUDA-core form walks; only the summation order
// differs.
//
// The visited set is a small epoch-tagged open-addressing hash in shared
// memory (ids below 2^24) that forgets (see BeamVisited), so its size does
// not grow with ef and the kernel keeps its occupancy.  A query that exceeds
// the step bound goes to the overflow list and is answered by the rerun pass.
#pragma once

#include <cuda_fp16.h>
#include <cuda_fp8.h>

#include "compressed_layout.cuh"
#include "search_kernel.cuh"
#include "search_wide.cuh"

namespace hg {
namespace sk {

constexpr uint32_t kBeamSteps = 1u << 16;  // bound of the layer-0 loop

__device__ __forceinline__ void mma_16816(float (&c)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                          uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t pack_half2(__half lo, __half hi) {
  return static_cast<uint32_t>(__half_as_ushort(lo)) | (static_cast<uint32_t>(__half_as_ushort(hi)) << 16);
}

// Thread t's A-fragment registers (half2) of half h of a 128-element row
// chunk: k-steps 4h .. 4h + 3 (registers 8h .. 8h + 7 of its stream).
template <int PREC>
__device__ __forceinline__ void load_rowhalf(const void* vq, uint32_t id, int t, int h, uint32_t (&a)[8]) {
  if (id == kNoId) {
#pragma unroll
    for (int j = 0; j < 8; ++j) a[j] = 0u;
    return;
  }
  if (PREC == 1) {
    const uint4* p = reinterpret_cast<const uint4*>(static_cast<const __half*>(vq) + static_cast<size_t>(id) * 128u);
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      const uint4 u = __ldg(p + 4 * (2 * h + i) + t);
      a[4 * i] = u.x;
      a[4 * i + 1] = u.y;
      a[4 * i + 2] = u.z;
      a[4 * i + 3] = u.w;
    }
  } else {
    const uint4* p = reinterpret_cast<const uint4*>(static_cast<const uint8_t*>(vq) + static_cast<size_t>(id) * 128u);
    const uint4 u = __ldg(p + 4 * h + t);
    const uint32_t w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
    for (int j = 0; j < 4; ++j) {
#pragma unroll
      for (int pr = 0; pr < 2; ++pr) {
        const __half2_raw r =
            __nv_cvt_fp8x2_to_halfraw2(static_cast<__nv_fp8x2_storage_t>((w[j] >> (16 * pr)) & 0xFFFFu), __NV_E4M3);
        a[2 * j + pr] = static_cast<uint32_t>(r.x) | (static_cast<uint32_t>(r.y) << 16);
      }
    }
  }
}

// The query as the B operand: lanes of quad row 0 hold the high FP16 part,
// quad row 1 the low part (q - hi), others zero; qs scales the query by a
// power of two so that its largest element lies in [2^13, 2^14).
struct BeamQuery {
  uint32_t b[16];
  float qn;       // |q|^2 of the prepared query (FP32)
  float unscale;  // 1 / qs
};

__device__ __forceinline__ void beam_load_query(BeamQuery& Q, const SearchParams& P, const float* raw, float inv,
                                                bool cosine, float* qst, int lane) {
  // lane l holds logical dims 4l .. 4l+3 for the reductions
  float v[4];
  float nrm = 0.0f, mx = 0.0f;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const uint32_t k = 4u * lane + i;
    float x = k < P.dim ? __ldg(raw + k) : 0.0f;
    if (cosine) x = __fmul_rn(x, inv);
    v[i] = x;
    nrm = __fmaf_rn(x, x, nrm);
    mx = fmaxf(mx, fabsf(x));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    nrm += __shfl_xor_sync(kFull, nrm, o);
    mx = fmaxf(mx, __shfl_xor_sync(kFull, mx, o));
  }
  Q.qn = nrm;
  int ex = 0;
  if (mx > 0.0f) frexpf(mx, &ex);  // mx = f 2^ex, f in [0.5, 1)
  const int sh = 14 - ex;         // mx 2^sh in [2^13, 2^14)
  const float qs = ldexpf(1.0f, sh);
  Q.unscale = ldexpf(1.0f, -sh);
  __syncwarp();
#pragma unroll
  for (int i = 0; i < 4; ++i) qst[4 * lane + i] = v[i] * qs;  // exact: a power of two
  __syncwarp();
  const int g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int s = 0; s < 8; ++s) {
#pragma unroll
    for (int hf = 0; hf < 2; ++hf) {
      const int k0 = 16 * s + 2 * t + 8 * hf;  // this lane's dims k0, k0 + 1 at k-step s
      const float x0 = qst[k0], x1 = qst[k0 + 1];
      const __half h0 = __float2half_rn(x0), h1 = __float2half_rn(x1);
      const __half l0 = __float2half_rn(x0 - __half2float(h0)), l1 = __float2half_rn(x1 - __half2float(h1));
      Q.b[2 * s + hf] = g == 0 ? pack_half2(h0, h1) : (g == 1 ? pack_half2(l0, l1) : 0u);
    }
  }
  __syncwarp();
}

// Distances of the rows fid[0..nf) into fdist[0..nf), 16 rows per
// tensor-core group.  Whole warp.
template <int PREC, bool L2>
__device__ __forceinline__ void beam_dists(const SearchParams& P, const BeamQuery& Q, const uint32_t* fid, int nf,
                                           float* fdist, int lane) {
  const int g = lane >> 2, t = lane & 3;
  const float2* aux = reinterpret_cast<const float2*>(P.vaux);
  for (int base = 0; base < nf; base += 16) {
    const int r0 = base + g, r1 = base + g + 8;
    const uint32_t id0 = r0 < nf ? fid[r0] : kNoId;
    const uint32_t id1 = r1 < nf ? fid[r1] : kNoId;
    float2 x0 = make_float2(1.0f, 0.0f), x1 = make_float2(1.0f, 0.0f);
    if (t == 0) {
      if (id0 != kNoId) x0 = __ldg(aux + id0);
      if (id1 != kNoId) x1 = __ldg(aux + id1);
    }
    float c[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      uint32_t a0[8], a1[8];
      load_rowhalf<PREC>(P.vq, id0, t, h, a0);
      load_rowhalf<PREC>(P.vq, id1, t, h, a1);
#pragma unroll
      for (int s = 0; s < 4; ++s)
        mma_16816(c, a0[2 * s], a1[2 * s], a0[2 * s + 1], a1[2 * s + 1], Q.b[8 * h + 2 * s], Q.b[8 * h + 2 * s + 1]);
    }
    if (t == 0) {
      const float d0 = (c[0] + c[1]) * Q.unscale, d1 = (c[2] + c[3]) * Q.unscale;
      if (r0 < nf) fdist[r0] = L2 ? Q.qn - 2.0f * x0.x * d0 + x0.y : 1.0f - x0.x * d0;
      if (r1 < nf) fdist[r1] = L2 ? Q.qn - 2.0f * x1.x * d1 + x1.y : 1.0f - x1.x * d1;
    }
  }
  __syncwarp();
}

// Per-warp visited set: an epoch-tagged open-addressing hash in shared
// memory (ids below 2^24).  It forgets: past 5/8 load the warp starts a new
// epoch and re-inserts the beam's ids.  A node visited before that and seen
// again costs one more distance and nothing else: if it left the beam, its
// key is worse than the worst kept key (which only improves) and is
// dropped; if it is still in the beam or the results, the merge finds the
// key there and drops the copy.
struct BeamVisited {
  uint32_t tag;
  uint32_t count;
  uint32_t resets;
  uint32_t H;  // slots this query uses (a power of two fixed by its own ef)
};

// true if id was not in the set (and is in it now); valid lanes only
__device__ __forceinline__ bool beam_visit(uint32_t* hash, const BeamVisited& V, uint32_t id) {
  const uint32_t key = V.tag | id;
  uint32_t p = (id * 0x9E3779B1u) >> (1 + __clz(V.H));
  for (uint32_t i = 0; i < V.H; ++i) {
    const uint32_t v = *reinterpret_cast<volatile const uint32_t*>(&hash[p]);
    if ((v & 0xFF000000u) != V.tag) {  // a slot of an earlier epoch: free
      const uint32_t old = atomicCAS(&hash[p], v, key);
      if (old == v) return true;
      if (old == key) return false;
      continue;
    }
    if (v == key) return false;
    p = (p + 1) & (V.H - 1u);
  }
  return false;  // unreachable below the 5/8 load limit
}

// Merge the c sorted new keys s[0..c) into the sorted src[0..len), writing
// the smallest cap keys to dst (merge path: every key's final place is its
// index plus its rank in the other list, so each lane places its keys
// independently); returns the new length and lowers *first to the rank the
// smallest new key took.  Keys are unique.
__device__ __forceinline__ int merge_path(const uint64_t* src, int len, uint64_t* dst, int cap, const uint64_t* s,
                                          int c, uint32_t* first, int lane) {
  int p0 = 0;
  if (lane < c) {
    const uint64_t v = s[lane];
    const int r = lower_bound(src, len, v);
    if (lane + r < cap) dst[lane + r] = v;
    p0 = r;
  }
  for (int i = lane; i < len; i += 32) {
    const uint64_t v = src[i];
    const int p = i + lower_bound(s, c, v);
    if (p < cap) dst[p] = v;
  }
  __syncwarp();
  *first = min(*first, static_cast<uint32_t>(__shfl_sync(kFull, p0, 0)));
  return min(len + c, cap);
}

// Merge stage[0..m) (unsorted, unique, every key better than the worst kept)
// into the sorted *cur (length len, capacity cap), 32 keys at a time through
// the ping-pong pair (*cur, *oth).  With dedup (the visited set forgot some
// nodes) keys whose (distance, id) is already held, or repeats in the chunk,
// are dropped first; the expanded flag (bit 0) is ignored there.
__device__ __forceinline__ int merge_keys(uint64_t*& cur, uint64_t*& oth, int len, int cap, uint64_t* st, int m,
                                          uint32_t* first, bool dedup, int lane) {
  for (int base = 0; base < m; base += 32) {
    int c = min(32, m - base);
    uint64_t v = lane < c ? st[base + lane] : kMaxKey;
    v = warp_sort32(v, lane);
    bool keep = lane < c;
    if (dedup) {
      const uint32_t plo = __shfl_up_sync(kFull, static_cast<uint32_t>(v), 1);
      const uint32_t phi = __shfl_up_sync(kFull, static_cast<uint32_t>(v >> 32), 1);
      const uint64_t prev = (static_cast<uint64_t>(phi) << 32) | plo;
      keep = keep && !(lane > 0 && (prev >> 1) == (v >> 1));
      if (keep) {
        const int r = lower_bound(cur, len, v & ~1ull);
        keep = !(r < len && (cur[r] >> 1) == (v >> 1));
      }
    }
    const uint32_t b = __ballot_sync(kFull, keep);
    c = __popc(b);
    __syncwarp();
    if (keep) st[base + __popc(b & ((1u << lane) - 1u))] = v;
    __syncwarp();
    if (c == 0) continue;
    len = merge_path(cur, len, oth, cap, st + base, c, first, lane);
    uint64_t* t = cur;
    cur = oth;
    oth = t;
  }
  return len;
}

__device__ __forceinline__ void prefetch_l2(const void* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

template <int PREC, bool L2, bool FILT, int ORD>
__global__ void __launch_bounds__(128, 6) beam_kernel(SearchParams P, const float* __restrict__ inv_norm) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  unsigned char* base = smem + static_cast<size_t>(wib) * beam_warp_bytes(P.H, P.R, FILT);
  uint32_t* hash = reinterpret_cast<uint32_t*>(base);
  uint64_t* const beamA = reinterpret_cast<uint64_t*>(base + 4u * P.H);
  uint64_t* const beamB = beamA + P.R;
  uint64_t* const resA = beamB + P.R;                 // FILT only
  uint64_t* const resB = resA + P.R;                  // FILT only
  uint64_t* const stage = FILT ? resB + P.R : resA;  // accepted keys
  uint64_t* const est = stage + 32 * kBeamMaxE;       // eligible accepted keys (FILT only)
  uint32_t* const fid = reinterpret_cast<uint32_t*>((FILT ? est : stage) + 32 * kBeamMaxE);
  float* const fdist = reinterpret_cast<float*>(fid + 32 * kBeamMaxE);
  for (uint32_t i = lane; i < P.H; i += 32) hash[i] = 0u;  // epoch 0: every slot free
  __syncwarp();

  const int E = static_cast<int>(min(max(P.lists_per_step, 1u), static_cast<uint32_t>(kBeamMaxE)));
  const size_t rstride = PREC == 1 ? 256u : 128u;  // bytes of a compressed row
  uint32_t nq = P.nq_dev ? min(*P.nq_dev, P.nq) : P.nq;
  if (P.lpt_sizes) {
    nq = 0;
    for (uint32_t b = 0; b < P.lpt_buckets; ++b) nq += P.lpt_sizes[b];
    nq = min(nq, P.nq);
  }
  uint32_t epoch = 0;
  BeamQuery Q;

  for (;;) {
    uint32_t item = 0;
    if (lane == 0) item = atomicAdd(P.work, 1u);
    item = __shfl_sync(kFull, item, 0);
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
    if (q >= P.nq) continue;
    const uint32_t k = P.kq ? P.kq[q] : P.k_all;
    uint32_t ef = P.efq ? P.efq[q] : P.ef_all;
    if (ef == 0) ef = P.ef_default;
    if (ef < k) ef = k;
    if (ef > P.R || k > P.k_stride || k == 0) {
      if (lane == 0) atomicExch(P.err, 1u);
      continue;
    }
    const int efi = static_cast<int>(ef);
    const uint32_t* fb = nullptr;
    if (FILT && P.fsel) {
      const int32_t f = P.fsel[q];
      if (f >= 0) fb = P.fbits[f];
    }
    if (++epoch == 256u) {  // 8-bit epochs: clear the hash every 255 queries
      for (uint32_t i = lane; i < P.H; i += 32) hash[i] = 0u;
      __syncwarp();
      epoch = 1;
    }
    BeamVisited V{epoch << 24, 0u, 0u, min(beam_hash_slots(ef), P.H)};
    const uint32_t hlimit = V.H / 8u * 5u;
    // the candidate beam's capacity: ef, or (filtered) a function of ef alone
    const int bcap = FILT ? min(static_cast<int>(P.R), (efi + 31) / 32 * 32) : efi;
    beam_load_query(Q, P, P.queries + static_cast<size_t>(q) * P.dim, inv_norm ? inv_norm[q] : 1.0f,
                    inv_norm != nullptr, fdist, lane);
    // traversal counters (lane 0 keeps them): upper lists / distances,
    // layer-0 lists / distances, steps
    uint32_t c_ul = 0, c_ud = 1, c_l = 0, c_d = 0, c_steps = 0;

    // ---- entry point + greedy descent (search_layer.cpp:29-56) on compressed rows ----
    uint32_t cur_id = P.entry;
    if (lane == 0) fid[0] = cur_id;
    __syncwarp();
    beam_dists<PREC, L2>(P, Q, fid, 1, fdist, lane);
    float cur_d = fdist[0];
    for (int lc = P.max_level; lc > 0; --lc) {
      bool changed = true;
      while (changed) {
        changed = false;
        const uint32_t* lst = P.up + static_cast<size_t>(__ldg(P.up_blk + cur_id) + (lc - 1)) * P.up_stride;
        const uint32_t id = static_cast<uint32_t>(lane) < P.M ? __ldg(lst + lane) : kNoId;  // M <= 32
        const uint32_t vm = __ballot_sync(kFull, id != kNoId);
        if (!vm) break;
        const int cnt = __popc(vm);
        const int pos = __popc(vm & ((1u << lane) - 1u));  // list order kept
        ++c_ul;
        c_ud += cnt;
        __syncwarp();
        if (id != kNoId) fid[pos] = id;
        __syncwarp();
        beam_dists<PREC, L2>(P, Q, fid, cnt, fdist, lane);
        const float d = id != kNoId ? fdist[pos] : __int_as_float(0x7f800000);
        const float m = warp_minf(d);
        if (m < cur_d) {
          const uint32_t hit = __ballot_sync(kFull, id != kNoId && d == m);
          cur_id = __shfl_sync(kFull, id, __ffs(hit) - 1);
          cur_d = m;
          changed = true;
        }
        __syncwarp();
      }
    }

    // ---- layer 0: beam search ----
    bool ovf = false;
    uint64_t* cur = beamA;
    uint64_t* oth = beamB;
    uint64_t* rcur = resA;
    uint64_t* roth = resB;
    if (lane == 0) {
      beam_visit(hash, V, cur_id);
      cur[0] = wkey(cur_d, cur_id);
    }
    V.count = 1;
    int blen = 1;
    int rlen = 0;
    if (FILT) {
      const bool e0 = bit_of(P.alive, cur_id) && (!fb || bit_of(fb, cur_id));
      if (e0) {
        if (lane == 0) rcur[0] = wkey(cur_d, cur_id);
        rlen = 1;
      }
    }
    __syncwarp();
    uint32_t hint = 0;
    for (uint32_t step = 0;; ++step) {
      if (step >= kBeamSteps) {
        ovf = true;
        break;
      }
      // worst accepted key: the ef-th result (the beam itself when unfiltered)
      const int rn = FILT ? rlen : blen;
      const uint64_t worst = rn >= efi ? ((FILT ? rcur : cur)[efi - 1] | 1ull) : kMaxKey;
      // 1. select the E best unexpanded entries not beyond the worst result
      uint32_t selv = kNoId;  // lane e holds the e-th selected id
      int nsel = 0;
      uint32_t next = hint;
      for (uint32_t b0 = hint & ~31u; b0 < static_cast<uint32_t>(blen) && nsel < E; b0 += 32) {
        const uint32_t i = b0 + lane;
        const bool live = i < static_cast<uint32_t>(blen);
        const uint64_t v = live ? cur[i] : kMaxKey;
        uint32_t bal = __ballot_sync(kFull, live && !(v & 1ull));
        uint32_t bey = 0;
        if (FILT) {
          bey = __ballot_sync(kFull, live && (v | 1ull) > worst);  // sorted: a suffix
          if (bey) bal &= (1u << (__ffs(bey) - 1)) - 1u;
        }
        const uint32_t myid = wkey_id(v);
        while (bal && nsel < E) {
          const int l = __ffs(bal) - 1;
          bal &= bal - 1;
          if (lane == l) cur[i] = v | 1ull;
          const uint32_t sid = __shfl_sync(kFull, myid, l);
          if (lane == nsel) selv = sid;
          ++nsel;
          next = b0 + static_cast<uint32_t>(l) + 1u;
        }
        if (bey) break;
      }
      hint = next;
      if (nsel == 0) break;
      ++c_steps;
      c_l += nsel;
      __syncwarp();
      // 2. the selected lists, loaded together
      uint32_t ids[kBeamMaxE];
#pragma unroll
      for (int e = 0; e < kBeamMaxE; ++e) {
        const uint32_t se = __shfl_sync(kFull, selv, e);
        ids[e] = (e < nsel && static_cast<uint32_t>(lane) < P.M0)
                     ? __ldg(P.l0 + static_cast<size_t>(se) * P.l0_stride + lane)
                     : kNoId;
      }
      // 3. visited test, fresh ids packed into fid (their rows prefetched to L2)
      int nf = 0;
#pragma unroll
      for (int e = 0; e < kBeamMaxE; ++e) {
        if (e >= nsel) break;
        const uint32_t id = ids[e];
        const bool valid = id != kNoId;
        const uint32_t vm = __ballot_sync(kFull, valid);
        if (V.count + static_cast<uint32_t>(__popc(vm)) > hlimit) {
          // forget: a new epoch holding the beam's ids and this step's fresh ids
          if (++epoch == 256u) {
            for (uint32_t i = lane; i < P.H; i += 32) hash[i] = 0u;
            epoch = 1;
          }
          V.tag = epoch << 24;
          ++V.resets;
          __syncwarp();
          for (int i = lane; i < blen; i += 32) beam_visit(hash, V, wkey_id(cur[i]));
          for (int i = lane; i < nf; i += 32) beam_visit(hash, V, fid[i]);
          V.count = static_cast<uint32_t>(blen + nf);
          __syncwarp();
        }
        bool first = valid;
        if (P.dedup && valid) first = (__ffs(__match_any_sync(vm, id)) - 1) == lane;
        const bool fresh = first && beam_visit(hash, V, id);
        __syncwarp();
        const uint32_t fm = __ballot_sync(kFull, fresh);
        if (fresh) {
          fid[nf + __popc(fm & ((1u << lane) - 1u))] = id;
          const unsigned char* row = static_cast<const unsigned char*>(P.vq) + static_cast<size_t>(id) * rstride;
          prefetch_l2(row);
          if (PREC == 1) prefetch_l2(row + 128);
        }
        nf += __popc(fm);
        V.count += __popc(fm);
      }
      __syncwarp();
      c_d += nf;
      if (nf == 0) continue;
      // 4. distances on the tensor cores
      beam_dists<PREC, L2>(P, Q, fid, nf, fdist, lane);
      // 5. keys better than the worst result enter the beam (and, if
      //    eligible, the results)
      int m = 0, ne = 0;
      for (int b0 = 0; b0 < nf; b0 += 32) {
        const int i = b0 + lane;
        uint64_t v = kMaxKey;
        bool keep = false, ok = false;
        if (i < nf) {
          const uint32_t id = fid[i];
          v = wkey(fdist[i], id);
          keep = v < worst;
          if (FILT) ok = keep && bit_of(P.alive, id) && (!fb || bit_of(fb, id));
        }
        const uint32_t bal = __ballot_sync(kFull, keep);
        if (keep) stage[m + __popc(bal & ((1u << lane) - 1u))] = v;
        m += __popc(bal);
        if (FILT) {
          const uint32_t be = __ballot_sync(kFull, ok);
          if (ok) est[ne + __popc(be & ((1u << lane) - 1u))] = v;
          ne += __popc(be);
        }
      }
      __syncwarp();
      if (FILT) {
        uint32_t unused = 0xFFFFFFFFu;
        rlen = merge_keys(rcur, roth, rlen, efi, est, ne, &unused, V.resets > 0, lane);
      }
      blen = merge_keys(cur, oth, blen, bcap, stage, m, &hint, V.resets > 0, lane);
    }
    if (ovf) {  // the rerun pass answers this query
      if (lane == 0) {
        const uint32_t o = atomicAdd(P.ovf_count, 1u);
        if (o < P.nq) P.ovf_list[o] = q;
      }
      __syncwarp();
      continue;
    }
    // ---- exact FP32 rerank of the best results, output ----
    const uint64_t* rarr = FILT ? rcur : cur;
    int s = FILT ? rlen : min(blen, efi);
    if (P.rerank_factor) {
      const uint64_t depth = max(32ull, static_cast<unsigned long long>(P.rerank_factor) * k);
      if (static_cast<uint64_t>(s) > depth) s = static_cast<int>(depth);
    }
    uint32_t* prow = P.pool_out + static_cast<size_t>(q) * P.pool_stride;
    for (int j = lane; j < s; j += 32) prow[j] = wkey_id(rarr[j]);
    if (lane == 0) P.pool_n[q] = static_cast<uint32_t>(s);
    __syncwarp();
    fused_rerank<typename ApproxDist<4, 16, PREC, ORD>::Exact, L2>(
        P.vecs, P.pd, P.dim, P.queries + static_cast<size_t>(q) * P.dim, inv_norm ? inv_norm[q] : 1.0f,
        inv_norm != nullptr, prow, s, oth, stage, static_cast<int>(P.R), lane);
    const int mk = s < static_cast<int>(k) ? s : static_cast<int>(k);
    QueryOut* row = static_cast<QueryOut*>(P.out) + static_cast<size_t>(q) * P.k_stride;
    for (uint32_t j = lane; j < P.k_stride; j += 32) {
      QueryOut o;
      if (static_cast<int>(j) < mk) {
        const uint64_t kk = oth[j];
        o.label = P.labels[static_cast<uint32_t>(kk)];
        o.dist = key_dist(kk);
      } else {
        o.label = ~0ull;
        o.dist = __int_as_float(0x7f800000);
      }
      o.zero = 0;
      row[j] = o;
    }
    if (P.nres && lane == 0) P.nres[q] = static_cast<uint32_t>(mk);
    if (P.counters && lane == 0) {
      unsigned long long* cp = P.counters + static_cast<size_t>(q) * kCounters;
      cp[0] = c_ul;
      cp[1] = c_ud;
      cp[2] = c_l;
      cp[3] = c_d;
      cp[4] = c_d + 1u;
      cp[5] = c_steps;
      cp[6] = static_cast<unsigned long long>(s);
      cp[7] = V.resets;
    }
    if (P.done) signal_done(P.done, q, lane);
    __syncwarp();
  }
}

template <int PREC, bool L2, bool FILT, int ORD>
cudaError_t beam_launch_t(const SearchParams& P, const float* inv, int blocks, int wpb, cudaStream_t st) {
  auto* fn = beam_kernel<PREC, L2, FILT, ORD>;
  cudaError_t e = open_smem_limit(reinterpret_cast<const void*>(fn));
  if (e != cudaSuccess) return e;
  fn<<<blocks, 32 * wpb, static_cast<size_t>(wpb) * beam_warp_bytes(P.H, P.R, FILT), st>>>(P, inv);
  return cudaGetLastError();
}

template <int PREC, bool L2, bool FILT, int ORD>
int beam_occupancy_t(int wpb, size_t smem) {
  int blocks = 0;
  auto* fn = beam_kernel<PREC, L2, FILT, ORD>;
  if (open_smem_limit(reinterpret_cast<const void*>(fn)) != cudaSuccess) return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, fn, 32 * wpb, smem) != cudaSuccess) return 0;
  return blocks;
}

template <int ORD>
cudaError_t beam_launch(const SearchParams& P, const float* inv, int blocks, int wpb, bool filt, cudaStream_t st) {
  if (P.pdc != 128) return cudaErrorInvalidValue;
  const bool fp8 = P.vscale != nullptr;
  if (P.metric == 0) {
    if (fp8) return filt ? beam_launch_t<2, true, true, ORD>(P, inv, blocks, wpb, st)
                         : beam_launch_t<2, true, false, ORD>(P, inv, blocks, wpb, st);
    return filt ? beam_launch_t<1, true, true, ORD>(P, inv, blocks, wpb, st)
                : beam_launch_t<1, true, false, ORD>(P, inv, blocks, wpb, st);
  }
  if (fp8) return filt ? beam_launch_t<2, false, true, ORD>(P, inv, blocks, wpb, st)
                       : beam_launch_t<2, false, false, ORD>(P, inv, blocks, wpb, st);
  return filt ? beam_launch_t<1, false, true, ORD>(P, inv, blocks, wpb, st)
              : beam_launch_t<1, false, false, ORD>(P, inv, blocks, wpb, st);
}

template <int ORD>
int beam_occupancy(int metric, int prec, int wpb, size_t smem, bool filt) {
  if (metric == 0) {
    if (prec == 2) return filt ? beam_occupancy_t<2, true, true, ORD>(wpb, smem)
                               : beam_occupancy_t<2, true, false, ORD>(wpb, smem);
    return filt ? beam_occupancy_t<1, true, true, ORD>(wpb, smem) : beam_occupancy_t<1, true, false, ORD>(wpb, smem);
  }
  if (prec == 2) return filt ? beam_occupancy_t<2, false, true, ORD>(wpb, smem)
                             : beam_occupancy_t<2, false, false, ORD>(wpb, smem);
  return filt ? beam_occupancy_t<1, false, true, ORD>(wpb, smem) : beam_occupancy_t<1, false, false, ORD>(wpb, smem);
}

}  // namespace sk
}  // namespace hg
