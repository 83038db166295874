// bf_mma.cu -- exact brute-force k-NN on the 5th-generation tensor cores.
//
// The reference scans every row with its SIMD distance kernel and keeps the
// k smallest (distance, label) pairs (src/brute_force.cpp:34-69).  Here the
// scan is a GEMM: queries (M = 128 per tile) times rows (N = 256 per tile)
// in FP16 with FP32 accumulation, tcgen05.mma issued by one thread, operands
// staged by TMA (128-byte swizzle, 4-stage mbarrier pipeline), the
// accumulator double-buffered in TMEM (2 x 256 columns) and read back by four
// epilogue warps (tcgen05.ld) that keep each query's candidates.
//
// Exactness.  For a query q and row x the GEMM gives s = |x|^2 - 2 q.x (L2)
// or -q.x (inner product / cosine), and the reference's distance d differs
// from s + |q|^2 (resp. 1 + s) by at most E(q): FP16 rounding of both
// operands (relative 2^-11, absolute 2^-25 below the FP16 normal range after
// power-of-two scaling), FP32 accumulation (bounded as sequential with
// truncation), the FP32 norm and the reference's own FP32 rounding.  Every
// row with s <= T + 2E, where T is the k-th smallest s, is kept; the true k
// nearest (ties included) are among them, and their exact distances are then
// computed in the reference's summation order and sorted by (distance, row).
// For integer data with |v| <= 2048, dim * max|q| * max|x| < 2^24 and
// dim * max(|q|, |x|)^2 < 2^24 the products, the GEMM sums and the norms are
// exact; every row whose true distance is below 2^24 then has s + |q|^2
// equal to the reference's distance, so E = 0 whenever the k-th smallest
// s + |q|^2 is below 2^24 (checked per query).  A query whose candidates do not fit the
// buffers is reported, and the caller answers that batch with the
// CUDA-core scan.
#include <cuda.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "bf_common.cuh"
#include "bf_mma.h"
#include "smem_limit.cuh"
#include "hnswgpu_device.h"

namespace hg::bfm {
namespace {

using namespace hg::bf;

constexpr int BM = 128;  // queries per tile (TMEM lanes)
constexpr int BN = 256;  // rows per tile (TMEM columns per accumulator)
constexpr int BK = 64;   // FP16 elements per K chunk: one 128-byte swizzle atom
constexpr int kStages = 4;
constexpr uint32_t kABytes = BM * BK * 2;
constexpr uint32_t kBBytes = BN * BK * 2;
// Epilogue warps per CTA: EPI = 8 (two per TMEM lane quarter, each over
// half of a tile's rows, chunks software-pipelined) for scans of few query
// tiles, EPI = 16 (four per quarter, a quarter of the rows each, 96
// registers) for many: warp 0 is the TMA producer, warp 1 issues the MMAs
// and owns TMEM, warps 2 .. EPI + 1 score.
template <int EPI>
struct Epi {
  static constexpr int kWarps = EPI;
  static constexpr uint32_t kParts = EPI / 4;           // column parts of a tile
  static constexpr uint32_t kPartCols = BN / kParts;    // tile rows per warp
  static constexpr uint32_t kPartChunks = kPartCols / 32;
  static constexpr int kThreads = 64 + 32 * EPI;
};
// scans of at least this many query tiles use the sixteen-warp epilogue
constexpr uint32_t kWideEpiTiles = 8;
constexpr uint32_t kTmemCols = 512;
constexpr size_t kSmem = kStages * (kABytes + kBBytes) + 1024;
constexpr uint32_t kOver = 0xFFFFFFFFu;
constexpr uint32_t kMaxPool = 4096;
constexpr uint32_t kMaxDim = 1024;
constexpr uint32_t kMaxK = 256;
constexpr uint64_t kWaitNs = 500ull * 1000 * 1000;  // bound of every pipeline wait

// instruction descriptor: D f32, A/B f16, both K-major, N = 256, M = 128
constexpr uint32_t kIdesc = (1u << 4) | (0u << 7) | (0u << 10) | (static_cast<uint32_t>(BN >> 3) << 17) |
                            (static_cast<uint32_t>(BM >> 4) << 24);

struct MmaParams {
  const float* xn;        // n_pad: |x|^2 (L2) or 0
  const uint32_t* allow;  // bits over rows or null
  const float* qc;        // nq_pad: s = xn + acc * qc
  const float* qm;        // nq_pad: selection margin 2E
  uint64_t* buf;          // (parts x splits) x nq x cap candidate keys: one set per tile part
  uint32_t* cnt;          // (2 x splits) x nq: candidates kept, or kOver
  uint32_t* err;          // [0] pipeline wait expired
  // per-query filters (routed graph queries): bits over rows of filter
  // fsel[q] (-1 none) instead of `allow`; tombstones over rows
  const uint32_t* const* allow_tab;
  const int32_t* fsel;
  const uint32_t* alive;
  // per query: the tightest bound any CTA has found so far (order-preserving
  // key bits, 0xFFFFFFFF none), shared by all splits of the query
  uint32_t* gkey;
  uint32_t n, nq, kchunks, cap, k, nbt, tiles_q, splits, tps;
  uint32_t trig;   // a lane's buffer is compacted once it could pass trig - 32 keys (<= cap)
  uint32_t trig0;  // the same for a sub-split's first compaction (its threshold starts at +inf)
  int l2;
  int lenient;  // keep the buffer of a query whose candidates overflow (approximate answer) instead of failing
  // bound pass: keep nothing; write each (tile part, query)'s smallest score
  // to mins[(parts * row tile + part) * nq_pad + q] (+inf if no row is allowed)
  int bound_pass;
  float* mins;
  uint32_t nq_pad;
  uint32_t tstep;  // row tiles taken: those with bt % tstep == 0 (the bound pass samples; 1 = all)
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ uint64_t globaltimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
// Wait for the phase of parity `parity` to complete; false once the time bound
// passes (the CTA's abort flag and the global error word are then set) or
// another role of the CTA gave up.
__device__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile uint32_t* abort_flag, uint32_t* err) {
  if (mbar_try(bar, parity)) return true;
  const uint64_t t0 = globaltimer();
  for (uint32_t i = 1;; ++i) {
    if (mbar_try(bar, parity)) return true;
    if ((i & 63u) == 0) {
      if (*abort_flag) return false;
      if (globaltimer() - t0 > kWaitNs) {
        *abort_flag = 1u;
        atomicExch(err, 1u);
        return false;
      }
    }
  }
}
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, uint32_t bar, int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
      : "memory");
}
// shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups 1024 B apart
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
  uint64_t d = static_cast<uint64_t>((saddr & 0x3FFFFu) >> 4);
  d |= static_cast<uint64_t>(1) << 16;            // leading byte offset (unused with this swizzle)
  d |= static_cast<uint64_t>(1024 >> 4) << 32;    // stride byte offset
  d |= static_cast<uint64_t>(1) << 46;            // descriptor version
  d |= static_cast<uint64_t>(2) << 61;            // 128-byte swizzle
  return d;
}
__device__ __forceinline__ void umma_f16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
          tmem_d),
      "l"(a), "l"(b), "r"(kIdesc), "r"(accumulate));
}
__device__ __forceinline__ void umma_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// tcgen05.ld without its wait: r may be read only after tmem_wait(r).
__device__ __forceinline__ void tmem_ld32_async(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
      "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
}

// Wait for this thread's TMEM loads.  r passes through the wait, so no read
// of it is scheduled above it.
__device__ __forceinline__ void tmem_wait(uint32_t (&r)[32]) {
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                 "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]),
                 "+r"(r[15]), "+r"(r[16]), "+r"(r[17]), "+r"(r[18]), "+r"(r[19]), "+r"(r[20]), "+r"(r[21]),
                 "+r"(r[22]), "+r"(r[23]), "+r"(r[24]), "+r"(r[25]), "+r"(r[26]), "+r"(r[27]), "+r"(r[28]),
                 "+r"(r[29]), "+r"(r[30]), "+r"(r[31])
               :
               : "memory");
}

__device__ __forceinline__ void sp_mma(float (&c)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0,
                                       uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// Packed FP32 pairs (sm_100+): each lane is the scalar op's IEEE result.
__device__ __forceinline__ float2 fma2_rn(float2 a, float2 b, float2 c) {
  unsigned long long pa, pb, pc, pd;
  asm("mov.b64 %0, {%1, %2};" : "=l"(pa) : "f"(a.x), "f"(a.y));
  asm("mov.b64 %0, {%1, %2};" : "=l"(pb) : "f"(b.x), "f"(b.y));
  asm("mov.b64 %0, {%1, %2};" : "=l"(pc) : "f"(c.x), "f"(c.y));
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(pd) : "l"(pa), "l"(pb), "l"(pc));
  float2 d;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(d.x), "=f"(d.y) : "l"(pd));
  return d;
}
__device__ __forceinline__ float2 mul2_rn(float2 a, float2 b) {
  unsigned long long pa, pb, pd;
  asm("mov.b64 %0, {%1, %2};" : "=l"(pa) : "f"(a.x), "f"(a.y));
  asm("mov.b64 %0, {%1, %2};" : "=l"(pb) : "f"(b.x), "f"(b.y));
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(pd) : "l"(pa), "l"(pb));
  float2 d;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(d.x), "=f"(d.y) : "l"(pd));
  return d;
}
// Three-input minimum; a NaN input is skipped, as fminf skips it.
__device__ __forceinline__ float min3f(float a, float b, float c) {
  float d;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
  return d;
}

__device__ __forceinline__ float dist_of_key_bits(uint32_t kb) {
  const uint32_t u = (kb & 0x80000000u) ? (kb & 0x7FFFFFFFu) : ~kb;
  return __uint_as_float(u);
}

// The warp compacts the candidate buffer of one of its lanes: a bound T with
// at least k and at most k + 32 keys of b[0..cnt) at or below it (at most k,
// i.e. the k-th smallest, when cnt <= 64; the exact k-th smallest, if the
// key bits allow no such bound) is found by
// bisection on the order-preserving key bits, then the keys within T + margin
// are kept.  The buffer (cnt <= 2 * kMaxK + 64) is held in registers, up to 18
// keys per lane; only the ceil(cnt / 32) register slots that hold keys are
// visited (a small k compacts at about a hundred keys: four slots).
__device__ __noinline__ uint32_t warp_compact(uint64_t* b, uint32_t cnt, uint32_t k, float margin, int lane,
                                              float* thr_out) {
  constexpr int kPer = (2 * static_cast<int>(kMaxK) + 64 + 31) / 32;
  const uint32_t jn = (cnt + 31u) >> 5;  // warp-uniform: the slots in use
  uint64_t v[kPer];
  uint32_t lo = 0xFFFFFFFFu, hi = 0u;
#pragma unroll
  for (int j = 0; j < kPer; ++j) {
    v[j] = ~0ull;
    if (static_cast<uint32_t>(j) < jn) {
      const uint32_t i = static_cast<uint32_t>(j) * 32u + static_cast<uint32_t>(lane);
      if (i < cnt) {
        v[j] = b[i];
        const uint32_t kb = static_cast<uint32_t>(v[j] >> 32);
        lo = min(lo, kb);
        hi = max(hi, kb);
      }
    }
  }
  lo = __reduce_min_sync(kFull, lo);
  hi = __reduce_max_sync(kFull, hi);
  uint32_t chi = cnt;  // keys at or below hi
  // a bound with up to k + 32 keys under it is good enough for a large
  // buffer; a small one (a first compaction) is cheap to cut to the k-th
  const uint32_t slack = cnt <= 64u ? 0u : 32u;
  while (lo < hi && chi > k + slack) {
    const uint32_t mid = lo + ((hi - lo) >> 1);
    uint32_t c = 0;
#pragma unroll
    for (int j = 0; j < kPer; ++j)
      if (static_cast<uint32_t>(j) < jn) c += static_cast<uint32_t>(v[j] >> 32) <= mid ? 1u : 0u;  // padding: ~0 > mid
    c = __reduce_add_sync(kFull, c);
    if (c >= k) {
      hi = mid;
      chi = c;
    } else {
      lo = mid + 1u;
    }
  }
  const float thr = __fadd_ru(dist_of_key_bits(hi), margin);
  __syncwarp();
  uint32_t w = 0;
#pragma unroll
  for (int j = 0; j < kPer; ++j) {
    if (static_cast<uint32_t>(j) >= jn) break;
    const uint32_t i = static_cast<uint32_t>(j) * 32u + static_cast<uint32_t>(lane);
    const bool keep = i < cnt && key_dist(v[j]) <= thr;
    const uint32_t bal = __ballot_sync(kFull, keep);
    if (keep) b[w + __popc(bal & ((1u << lane) - 1u))] = v[j];
    w += __popc(bal);
  }
  __syncwarp();
  *thr_out = thr;
  return w;
}

template <int EPI>
__global__ void __launch_bounds__(Epi<EPI>::kThreads, 1)
    bf_mma_kernel(const __grid_constant__ CUtensorMap map_q, const __grid_constant__ CUtensorMap map_x, MmaParams P) {
  constexpr int kEpiWarps = Epi<EPI>::kWarps;
  constexpr uint32_t kParts = Epi<EPI>::kParts, kPartCols = Epi<EPI>::kPartCols;
  constexpr uint32_t kPartChunks = Epi<EPI>::kPartChunks;
  extern __shared__ unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bars[2 * kStages + 5];
  __shared__ uint32_t tmem_slot;
  __shared__ volatile uint32_t abort_flag;
  unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t{1023});
  const uint32_t sbase = smem_u32(smem);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  auto sA = [&](int s) { return sbase + static_cast<uint32_t>(s) * kABytes; };
  auto sB = [&](int s) { return sbase + kStages * kABytes + static_cast<uint32_t>(s) * kBBytes; };
  auto full = [&](int s) { return smem_u32(&bars[s]); };
  auto empty = [&](int s) { return smem_u32(&bars[kStages + s]); };
  auto tfull = [&](int b) { return smem_u32(&bars[2 * kStages + b]); };
  auto tempty = [&](int b) { return smem_u32(&bars[2 * kStages + 2 + b]); };
  const uint32_t mdone = smem_u32(&bars[2 * kStages + 4]);

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(full(s), 1);
      mbar_init(empty(s), 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(tfull(b), 1);
      mbar_init(tempty(b), kEpiWarps);
    }
    mbar_init(mdone, 1);
    abort_flag = 0u;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;
  const uint32_t items = P.tiles_q * P.splits;

  if (warp == 0) {
    if (lane == 0) {
      // ---- TMA producer: query chunk + row chunk per stage ----
      uint32_t stage = 0, phase = 0;
      uint32_t issued_mask = 0, parity_mask = 0;  // per stage: a load was issued, parity of the last one
      bool ok = true;
      for (uint32_t item = blockIdx.x; ok && item < items; item += gridDim.x) {
        const uint32_t qt = item % P.tiles_q, sp = item / P.tiles_q;
        const uint32_t b0 = sp * P.tps, b1 = min(P.nbt, b0 + P.tps);
        for (uint32_t bt = (b0 + P.tstep - 1) / P.tstep * P.tstep; ok && bt < b1; bt += P.tstep) {
          for (uint32_t kc = 0; kc < P.kchunks; ++kc) {
            if (!mbar_wait(empty(stage), phase ^ 1u, &abort_flag, P.err)) {
              ok = false;
              break;
            }
            mbar_expect_tx(full(stage), kABytes + kBBytes);
            tma_load_2d(sA(stage), &map_q, full(stage), static_cast<int>(kc * BK), static_cast<int>(qt * BM));
            tma_load_2d(sB(stage), &map_x, full(stage), static_cast<int>(kc * BK), static_cast<int>(bt * BN));
            issued_mask |= 1u << stage;
            parity_mask = (parity_mask & ~(1u << stage)) | (phase << stage);
            if (++stage == kStages) {
              stage = 0;
              phase ^= 1u;
            }
          }
        }
      }
      // every copy issued has landed before the CTA exits (bounded)
      for (int st = 0; st < kStages; ++st) {
        if (!((issued_mask >> st) & 1u)) continue;
        const uint64_t t0 = globaltimer();
        while (!mbar_try(full(st), (parity_mask >> st) & 1u) && globaltimer() - t0 < kWaitNs) {
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // ---- MMA issuer ----
      uint32_t stage = 0, phase = 0, acc_i = 0;
      bool ok = true;
      for (uint32_t item = blockIdx.x; ok && item < items; item += gridDim.x) {
        const uint32_t sp = item / P.tiles_q;
        const uint32_t b0 = sp * P.tps, b1 = min(P.nbt, b0 + P.tps);
        for (uint32_t bt = (b0 + P.tstep - 1) / P.tstep * P.tstep; ok && bt < b1; bt += P.tstep, ++acc_i) {
          const uint32_t ab = acc_i & 1u, aph = (acc_i >> 1) & 1u;
          if (!mbar_wait(tempty(ab), aph ^ 1u, &abort_flag, P.err)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t d = tmem + ab * BN;
          for (uint32_t kc = 0; kc < P.kchunks; ++kc) {
            if (!mbar_wait(full(stage), phase, &abort_flag, P.err)) {
              ok = false;
              break;
            }
            tc_fence_after();
            const uint64_t a = sw128_desc(sA(stage)), b = sw128_desc(sB(stage));
#pragma unroll
            for (uint32_t kk = 0; kk < BK / 16; ++kk)  // K = 16 per MMA: +32 bytes in the swizzle atom
              umma_f16(d, a + 2u * kk, b + 2u * kk, (kc | kk) != 0u ? 1u : 0u);
            umma_commit(empty(stage));  // frees the stage once these MMAs have read it
            if (++stage == kStages) {
              stage = 0;
              phase ^= 1u;
            }
          }
          if (ok) umma_commit(tfull(ab));
        }
      }
      // all MMAs of this thread have completed before TMEM is released (bounded)
      umma_commit(mdone);
      const uint64_t t0 = globaltimer();
      while (!mbar_try(mdone, 0u) && globaltimer() - t0 < kWaitNs) {
      }
    }
  } else {
    // ---- epilogue: one query per thread (TMEM lane); a warp scores one part
    // of a tile's 256 rows, chunks kPartChunks * part .. kPartChunks *
    // (part + 1) - 1, keeping its own candidate buffers (sub-split kParts *
    // split + part) ----
    const uint32_t quarter = static_cast<uint32_t>(warp & 3);
    const uint32_t part = static_cast<uint32_t>(warp - 2) / 4u;
    const uint32_t c_begin = part * kPartChunks, c_end = c_begin + kPartChunks;
    const uint32_t row_in_tile = quarter * 32u + static_cast<uint32_t>(lane);
    uint32_t acc_i = 0;
    bool ok = true;
    for (uint32_t item = blockIdx.x; ok && item < items; item += gridDim.x) {
      const uint32_t qt = item % P.tiles_q, sp = item / P.tiles_q;
      const uint32_t b0 = sp * P.tps, b1 = min(P.nbt, b0 + P.tps);
      const uint32_t q = qt * BM + row_in_tile;
      const bool live_q = q < P.nq;
      const int32_t fq = (P.fsel && live_q) ? P.fsel[q] : -1;
      const uint32_t* allow_q = P.fsel ? (fq >= 0 ? P.allow_tab[fq] : nullptr) : P.allow;
      const float cq = P.qc[q];
      const float margin = P.qm[q];
      const uint32_t sub = kParts * sp + part;
      uint64_t* bufp = P.buf + (static_cast<size_t>(sub) * P.nq + (live_q ? q : 0)) * P.cap;
      uint32_t cnt = 0;
      uint32_t lim = P.trig0;  // compaction point: the threshold tightens early
      // the bound pass keeps no row: no score is at or below -inf
      float thr = P.bound_pass ? -__int_as_float(0x7f800000) : __int_as_float(0x7f800000);
      bool over = false;
      for (uint32_t bt = (b0 + P.tstep - 1) / P.tstep * P.tstep; bt < b1; bt += P.tstep, ++acc_i) {
        const uint32_t ab = acc_i & 1u, aph = (acc_i >> 1) & 1u;
        float tmin = __int_as_float(0x7f800000);  // bound pass: the part's smallest score
        if (bt + P.tstep < b1 && lane < static_cast<int>(kPartCols / 32))  // the next tile's row norms of this part into L1
          asm volatile("prefetch.global.L1 [%0];" ::"l"(P.xn + (bt + P.tstep) * BN + part * kPartCols + lane * 32u));
        // the bound of the other splits of this query (a split's k-th
        // smallest + the margin bounds the k-th over all rows from above)
        if (live_q && !over && !P.bound_pass) {
          const uint32_t gk = *reinterpret_cast<volatile const uint32_t*>(P.gkey + q);
          if (gk != 0xFFFFFFFFu) thr = fminf(thr, dist_of_key_bits(gk));
        }
        // one lane waits, the warp follows its answer (tcgen05.ld needs the whole warp)
        int got = 0;
        if (lane == 0) got = mbar_wait(tfull(ab), aph, &abort_flag, P.err) ? 1 : 0;
        if (!__shfl_sync(kFull, got, 0)) {
          ok = false;
          break;
        }
        tc_fence_after();
        const uint32_t taddr = tmem + ((quarter * 32u) << 16) + ab * BN;
        auto fetch = [&](uint32_t ch, uint32_t (&r)[32], uint32_t& valid) {
          tmem_ld32_async(taddr + ch * 32u, r);
          const uint32_t j0 = bt * BN + ch * 32u;
          valid = 0u;
          if (j0 < P.n && live_q && !over) {  // padding rows of the last tile stay masked
            valid = P.n - j0 >= 32u ? 0xFFFFFFFFu : ((1u << (P.n - j0)) - 1u);
            if (allow_q) valid &= __ldg(allow_q + (j0 >> 5));
            if (P.alive) valid &= __ldg(P.alive + (j0 >> 5));
          }
        };
        auto score = [&](uint32_t ch, const uint32_t (&r)[32], uint32_t valid) {
          // the chunk's row norms: the same 128 bytes for the whole warp, and
          // for the CTA's other warps on these rows (L1)
          float xs[32];
          {
            const float4* x4 = reinterpret_cast<const float4*>(P.xn + bt * BN + ch * 32u);  // < n_pad
#pragma unroll
            for (int v = 0; v < 8; ++v) {
              const float4 t = __ldg(x4 + v);
              xs[4 * v] = t.x;
              xs[4 * v + 1] = t.y;
              xs[4 * v + 2] = t.z;
              xs[4 * v + 3] = t.w;
            }
          }
          const uint32_t j0 = bt * BN + ch * 32u;
          if (over) valid = 0u;  // set by a compaction of an earlier chunk
          float sv[32];  // two rows per packed FP32 instruction (each lane rounded as a scalar op)
#pragma unroll
          for (int c = 0; c < 32; c += 2) {
            const float2 v = P.l2 ? fma2_rn(make_float2(__uint_as_float(r[c]), __uint_as_float(r[c + 1])),
                                            make_float2(cq, cq), make_float2(xs[c], xs[c + 1]))
                                  : mul2_rn(make_float2(__uint_as_float(r[c]), __uint_as_float(r[c + 1])),
                                            make_float2(cq, cq));
            sv[c] = v.x;
            sv[c + 1] = v.y;
          }
          if (valid != 0xFFFFFFFFu) {  // masked rows become NaN: never <= thr, skipped by min
#pragma unroll
            for (int c = 0; c < 32; ++c)
              if (!((valid >> c) & 1u)) sv[c] = __int_as_float(0x7fffffff);
          }
          float g8[4];  // minima of the four 8-row groups (three-input min)
#pragma unroll
          for (int g = 0; g < 4; ++g) {
            const float* v = sv + 8 * g;
            g8[g] = min3f(min3f(v[0], v[1], v[2]), min3f(v[3], v[4], v[5]), fminf(v[6], v[7]));
          }
          const float mn = min3f(g8[0], g8[1], fminf(g8[2], g8[3]));
          tmin = fminf(tmin, mn);
          if (mn <= thr) {  // rare once the threshold has settled
#pragma unroll
            for (int g = 0; g < 4; ++g) {
              if (g8[g] <= thr) {  // only the groups holding a passing row
#pragma unroll
                for (int c = 8 * g; c < 8 * g + 8; ++c)
                  if (sv[c] <= thr) bufp[cnt++] = (static_cast<uint64_t>(okey(sv[c])) << 32) | (j0 + c);
              }
            }
          }
          // room for the next chunk: compact the lanes that are nearly full
          uint32_t need = __ballot_sync(kFull, cnt + 32u > lim);
          while (need) {
            const int L = __ffs(need) - 1;
            need &= need - 1;
            uint64_t* lb = reinterpret_cast<uint64_t*>(__shfl_sync(kFull, reinterpret_cast<unsigned long long>(bufp), L));
            const uint32_t lc = __shfl_sync(kFull, cnt, L);
            const float lm = __shfl_sync(kFull, margin, L);
            float lthr;
            const uint32_t kept = warp_compact(lb, lc, P.k, lm, lane, &lthr);
            if (lane == L) {
              cnt = kept;
              thr = fminf(thr, lthr);  // both bound the k-th: keep the tighter
              lim = min(P.cap, max(P.trig, cnt + 64u));  // no compaction again before 32 new keys
              if (cnt + 32u > P.cap) {  // the margin keeps too many rows: give this query up
                over = true;
                thr = -__int_as_float(0x7f800000);
              } else {
                atomicMin(P.gkey + q, okey(lthr));  // publish this split's bound
              }
            }
          }
        };
        // tcgen05.ld / wait::ld are .sync.aligned: the warp is converged at each
        if constexpr (kPartChunks >= 4) {
          // two warps per scheduler: the TMEM load and the filter and
          // tombstone words of chunk ch + 1 are in flight while chunk ch is
          // scored
          uint32_t ra[32], rb[32];
          uint32_t va = 0, vb = 0;
          __syncwarp();
          fetch(c_begin, ra, va);
          tmem_wait(ra);
#pragma unroll 1
          for (uint32_t ch = c_begin; ch < c_end; ch += 2) {
            __syncwarp();
            fetch(ch + 1, rb, vb);
            score(ch, ra, va);
            __syncwarp();
            tmem_wait(rb);
            if (ch + 2 < c_end) fetch(ch + 2, ra, va);
            score(ch + 1, rb, vb);
            __syncwarp();
            if (ch + 2 < c_end) tmem_wait(ra);
          }
        } else {
          // four warps per scheduler hide the loads; one chunk in registers
#pragma unroll 1
          for (uint32_t ch = c_begin; ch < c_end; ++ch) {
            __syncwarp();
            uint32_t ra[32];
            uint32_t va = 0;
            fetch(ch, ra, va);
            tmem_wait(ra);
            score(ch, ra, va);
          }
        }
        __syncwarp();
        tc_fence_before();
        if (lane == 0) mbar_arrive(tempty(ab));
        if (P.bound_pass)
          P.mins[(static_cast<uint64_t>(kParts) * (bt / P.tstep) + part) * P.nq_pad + qt * BM + row_in_tile] = tmin;
      }
      if (ok && live_q && !P.bound_pass) P.cnt[static_cast<size_t>(sub) * P.nq + q] = (over && !P.lenient) ? kOver : cnt;
    }
  }
  __syncwarp();
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
  }
}

// ---------------------------------------------------------------------------
// rows: bound constants, FP16 copy and squared norms
// ---------------------------------------------------------------------------
struct RowStats {
  uint32_t max_abs_bits, max_l1_bits, max_l2_bits, all_int;
};

__global__ void row_stats_kernel(const float* __restrict__ rows, uint32_t n, uint32_t dim, uint32_t dp, RowStats* st) {
  const uint64_t r = (static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (r >= n) return;
  float mx = 0.0f;
  double l1 = 0.0, l2 = 0.0;
  bool isint = true;
  for (uint32_t i = lane; i < dim; i += 32) {
    const float v = rows[r * dp + i];
    const float a = fabsf(v);
    mx = fmaxf(mx, a);
    l1 += a;
    l2 += static_cast<double>(v) * v;
    isint = isint && v == rintf(v) && a <= 2048.0f;
  }
  for (int o = 16; o > 0; o >>= 1) {
    mx = fmaxf(mx, __shfl_xor_sync(kFull, mx, o));
    l1 += __shfl_xor_sync(kFull, l1, o);
    l2 += __shfl_xor_sync(kFull, l2, o);
  }
  isint = __all_sync(kFull, isint);
  if (lane == 0) {
    atomicMax(&st->max_abs_bits, __float_as_uint(mx));
    atomicMax(&st->max_l1_bits, __float_as_uint(__double2float_ru(l1)));
    atomicMax(&st->max_l2_bits, __float_as_uint(__double2float_ru(sqrt(l2))));
    if (!isint) atomicAnd(&st->all_int, 0u);
  }
}

__global__ void encode_rows_kernel(const float* __restrict__ rows, uint32_t n, uint32_t n_pad, uint32_t dim,
                                   uint32_t dp, uint32_t kp, float sigma, int l2, __half* __restrict__ x16,
                                   float* __restrict__ xn) {
  const uint64_t r = (static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (r >= n_pad) return;
  float ss = 0.0f;
  for (uint32_t i = lane; i < kp; i += 32) {
    const float v = (r < n && i < dim) ? rows[r * dp + i] : 0.0f;
    x16[r * kp + i] = __float2half_rn(__fmul_rn(v, sigma));
    ss = __fmaf_rn(v, v, ss);
  }
  for (int o = 16; o > 0; o >>= 1) ss = __fadd_rn(ss, __shfl_xor_sync(kFull, ss, o));
  if (lane == 0) xn[r] = (l2 && r < n) ? ss : 0.0f;
}

// ---------------------------------------------------------------------------
// queries: FP16 copy, scale and selection margin
// ---------------------------------------------------------------------------
struct DataBound {
  float sigma_x, x2, x1, xm;
  int all_int;
};

__global__ void prep_queries_kernel(const float* __restrict__ raw, const float* __restrict__ inv, uint32_t nq,
                                    uint32_t nq_pad, uint32_t dim, uint32_t kp, int l2, DataBound db,
                                    __half* __restrict__ q16, float* __restrict__ qc, float* __restrict__ qm,
                                    float* __restrict__ qq) {
  const uint64_t q = (static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (q >= nq_pad) return;
  const bool live = q < nq;
  const float iv = (live && inv) ? inv[q] : 1.0f;
  float mx = 0.0f;
  double l1 = 0.0, l2s = 0.0;
  bool isint = true;
  for (uint32_t i = lane; i < dim; i += 32) {
    float v = live ? raw[q * dim + i] : 0.0f;
    if (inv) v = __fmul_rn(v, iv);
    const float a = fabsf(v);
    mx = fmaxf(mx, a);
    l1 += a;
    l2s += static_cast<double>(v) * v;
    isint = isint && v == rintf(v) && a <= 2048.0f;
  }
  for (int o = 16; o > 0; o >>= 1) {
    mx = fmaxf(mx, __shfl_xor_sync(kFull, mx, o));
    l1 += __shfl_xor_sync(kFull, l1, o);
    l2s += __shfl_xor_sync(kFull, l2s, o);
  }
  isint = __all_sync(kFull, isint);
  const double d = static_cast<double>(dim);
  const double qn = sqrt(l2s) * (1.0 + 1e-12);
  const double mq = mx;
  const bool exact = db.all_int && isint && d * mq * db.xm < 16777216.0 && d * mq * mq < 16777216.0 &&
                     d * static_cast<double>(db.xm) * db.xm < 16777216.0;
  float sigma_q = 1.0f;
  if (!exact && mx > 0.0f) {
    int e;
    frexpf(mx, &e);                 // mx < 2^e
    sigma_q = ldexpf(1.0f, 14 - e);  // mx * sigma_q in [2^13, 2^14)
  }
  for (uint32_t i = lane; i < kp; i += 32) {
    float v = (live && i < dim) ? raw[q * dim + i] : 0.0f;
    if (inv) v = __fmul_rn(v, iv);
    q16[q * kp + i] = __float2half_rn(__fmul_rn(v, sigma_q));
  }
  if (lane != 0) return;
  const float unscale = 1.0f / (sigma_q * db.sigma_x);  // a power of two
  qc[q] = (l2 ? -2.0f : -1.0f) * unscale;
  qq[q] = exact ? static_cast<float>(l2 ? l2s : 1.0) : -1.0f;  // exact: |q|^2 (L2) or 1 (IP), else -1
  if (exact) {
    qm[q] = 0.0f;
    return;
  }
  // error bound E of s against the reference distance; the margin is 2 * (2E)
  const double u = 1.0 / 2048.0, p23 = 1.0 / 8388608.0, p24 = p23 / 2.0;
  const double c1 = 2.0 * u + u * u + (d + 2.0) * p23 * (1.0 + 2.0 * u + u * u);
  const double sub = 1.01 * (1.0 / 33554432.0) * (l1 / db.sigma_x + db.x1 / sigma_q) + d * 1e-15;
  const double edot = c1 * qn * db.x2 + sub;
  const double gam = (d + 2.0) * p24 * 1.01;
  double e;
  if (l2) {
    e = 2.0 * edot + gam * db.x2 * db.x2 + p23 * (db.x2 * db.x2 + 2.0 * qn * db.x2) +
        (2.0 * p23 + gam) * (qn + db.x2) * (qn + db.x2) + gam * qn * qn;
  } else {
    e = edot + gam * qn * db.x2 + 2.0 * p23 * (1.0 + qn * db.x2);
  }
  qm[q] = __double2float_ru(4.0 * e);
}

// ---------------------------------------------------------------------------
// per query, one CTA: the k-th smallest over the splits by a 4-pass radix
// select (8-bit digits of the order-preserving key bits), survivors within
// the margin.  The pool's order does not matter (the rerank sorts it).  The
// candidates are read 5-7 times by 256 threads; a warp bisecting the key
// bits read them about 34 times, which dominated scans split many ways
// (few queries over many rows).  The splits' counts are turned into offsets
// in shared memory first, so each pass walks the candidates of all splits
// as one flat range (a split is found by binary search) instead of one
// split after another.
// ---------------------------------------------------------------------------
constexpr int kSelThreads = 256;
constexpr uint32_t kSelMaxSplits = 1024;

// kq: per-query k (indexed through qlist when given), or null for k.
// bound_out (non-null): only the bound -- the order-preserving key of the
// k-th smallest score plus the margin, or +inf's key with at most k
// candidates -- is written per query; no pool.
__global__ void __launch_bounds__(kSelThreads) select_cta_kernel(
    const uint64_t* __restrict__ buf, const uint32_t* __restrict__ cnt, const float* __restrict__ qm,
    const float* __restrict__ qq, uint32_t nq, uint32_t splits, uint32_t cap, uint32_t k,
    uint32_t* __restrict__ pool, uint32_t pool_cap, uint32_t* __restrict__ pool_n, uint32_t* __restrict__ err,
    int lenient, const uint32_t* __restrict__ kq, const uint32_t* __restrict__ qlist,
    uint32_t* __restrict__ bound_out) {
  __shared__ uint32_t hist[256];
  __shared__ uint32_t wsum[kSelThreads / 32];
  __shared__ uint32_t soff[kSelMaxSplits + 1];
  __shared__ uint32_t sh_over, sh_bucket, sh_before, sh_count, sh_w;
  const uint32_t q = blockIdx.x;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  if (kq) k = kq[qlist ? qlist[q] : q];
  if (t == 0) {
    sh_over = 0u;
    sh_w = 0u;
  }
  __syncthreads();
  {
    // thread t owns splits 4t .. 4t + 3: counts, then an exclusive scan
    constexpr int kPer = kSelMaxSplits / kSelThreads;
    uint32_t c[kPer], sum = 0;
    bool ov = false;
#pragma unroll
    for (int i = 0; i < kPer; ++i) {
      const uint32_t sp = static_cast<uint32_t>(kPer * t + i);
      c[i] = 0u;
      if (sp < splits) {
        const uint32_t v = cnt[static_cast<size_t>(sp) * nq + q];
        if (v == kOver) ov = true;
        else c[i] = min(v, cap);
      }
      sum += c[i];
    }
    if (ov) atomicOr(&sh_over, 1u);
    uint32_t incl = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t u = __shfl_up_sync(kFull, incl, o);
      if (lane >= o) incl += u;
    }
    if (lane == 31) wsum[warp] = incl;
    __syncthreads();
    uint32_t base = 0;
    for (int w2 = 0; w2 < warp; ++w2) base += wsum[w2];
    uint32_t run = base + incl - sum;
#pragma unroll
    for (int i = 0; i < kPer; ++i) {
      soff[kPer * t + i] = run;
      run += c[i];
    }
    if (t == kSelThreads - 1) soff[kSelMaxSplits] = run;
  }
  __syncthreads();
  if (sh_over) {
    if (t == 0) {
      if (bound_out) {
        bound_out[q] = okey(__int_as_float(0x7f800000));
      } else {
        pool_n[q] = 0;
        atomicAdd(err + 1, 1u);
      }
    }
    return;
  }
  const uint32_t total = soff[kSelMaxSplits];
  // Up to kSelThreads * kSelReg candidates are read once into registers
  // (thread t holds candidates t, t + 256, ...), and every pass runs over
  // those; more are re-read from the buffers by each pass.
  constexpr int kSelReg = 16;
  const bool in_regs = total <= static_cast<uint32_t>(kSelThreads * kSelReg);
  uint64_t kv[kSelReg];
  if (in_regs) {
    uint32_t sp = 0;  // the split holding candidate i: soff[sp] <= i < soff[sp + 1]
#pragma unroll
    for (int j = 0; j < kSelReg; ++j) {
      const uint32_t i = static_cast<uint32_t>(t + j * kSelThreads);
      kv[j] = ~0ull;
      if (i < total) {
        while (soff[sp + 1] <= i) ++sp;
        kv[j] = buf[(static_cast<size_t>(sp) * nq + q) * cap + (i - soff[sp])];
      }
    }
  }
  auto for_each = [&](auto&& f) {
    if (in_regs) {
#pragma unroll
      for (int j = 0; j < kSelReg; ++j)
        if (static_cast<uint32_t>(t + j * kSelThreads) < total) f(kv[j]);
      return;
    }
    for (uint32_t i = t; i < total; i += kSelThreads) {
      uint32_t lo = 0, hi = splits;  // the split sp with soff[sp] <= i < soff[sp + 1]
      while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (soff[mid] <= i) lo = mid;
        else hi = mid;
      }
      f(buf[(static_cast<size_t>(lo) * nq + q) * cap + (i - soff[lo])]);
    }
  };
  // block-wide count of keys whose bits are <= kb
  auto count_le = [&](uint32_t kb) {
    __syncthreads();
    if (t == 0) sh_count = 0u;
    __syncthreads();
    uint32_t c = 0;
    for_each([&](uint64_t v) { c += static_cast<uint32_t>(v >> 32) <= kb ? 1u : 0u; });
    if (c) atomicAdd(&sh_count, c);
    __syncthreads();
    return sh_count;
  };
  // the r-th smallest (1-based, r <= total) key bits
  auto radix_select = [&](uint32_t r) {
    uint32_t prefix = 0u, pmask = 0u;
    for (int shift = 24; shift >= 0; shift -= 8) {
      hist[t] = 0u;  // kSelThreads == 256 bins
      __syncthreads();
      for_each([&](uint64_t v) {
        const uint32_t kb = static_cast<uint32_t>(v >> 32);
        if ((kb & pmask) == prefix) atomicAdd(&hist[(kb >> shift) & 255u], 1u);
      });
      __syncthreads();
      // inclusive scan of the 256 bins: within warps, then across them
      const uint32_t h = hist[t];
      uint32_t incl = h;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t u = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += u;
      }
      if (lane == 31) wsum[warp] = incl;
      __syncthreads();
      uint32_t base = 0;
      for (int w2 = 0; w2 < warp; ++w2) base += wsum[w2];
      incl += base;
      const uint32_t excl = incl - h;
      if (excl < r && r <= incl) {  // exactly one bin
        sh_bucket = static_cast<uint32_t>(t);
        sh_before = excl;
      }
      __syncthreads();
      prefix |= sh_bucket << shift;
      pmask |= 0xFFu << shift;
      r -= sh_before;
      __syncthreads();
    }
    return prefix;
  };
  float thr = __int_as_float(0x7f800000);
  if (bound_out) {
    if (total > k) thr = __fadd_ru(dist_of_key_bits(radix_select(k)), qm[q]);
    if (t == 0) bound_out[q] = okey(thr);
    return;
  }
  if (total > k) {
    const float T = dist_of_key_bits(radix_select(k));
    thr = __fadd_ru(T, qm[q]);
    if (lenient && count_le(okey(thr)) > pool_cap) {
      // too many survivors for the pool: keep the pool_cap smallest (approximate)
      const uint32_t lo2 = radix_select(pool_cap);
      thr = dist_of_key_bits(lo2);
      if (count_le(lo2) > pool_cap) thr = nextafterf(thr, -__int_as_float(0x7f800000));  // ties at the edge: drop them
    }
    // exact mode holds while the k-th distance is below 2^24 (where the
    // reference's own sum is still exact); past it the scan answers
    if (!lenient && qq[q] >= 0.0f && static_cast<double>(T) + qq[q] >= 16777216.0) {
      if (t == 0) {
        pool_n[q] = 0;
        atomicAdd(err + 1, 1u);
      }
      return;
    }
  }
  __syncthreads();
  for_each([&](uint64_t v) {
    if (key_dist(v) <= thr) {
      const uint32_t pos = atomicAdd(&sh_w, 1u);
      if (pos < pool_cap) pool[static_cast<size_t>(q) * pool_cap + pos] = static_cast<uint32_t>(v);
    }
  });
  __syncthreads();
  if (t == 0) {
    const uint32_t w = sh_w;
    if (w > pool_cap) {
      pool_n[q] = lenient ? pool_cap : 0;
      if (!lenient) atomicAdd(err + 1, 1u);
    } else {
      pool_n[q] = w;
    }
  }
}


// ---------------------------------------------------------------------------
// exact distances of the survivors in the reference order, sorted, first k
// ---------------------------------------------------------------------------
// Where rerank_kernel writes query q's row: out row out_index[q] (or q) with
// stride k_stride, the first min(m, k of that row) entries valid, then the
// row's done flag (system-scope fence first) when `done` is given.
struct OutMap {
  const uint32_t* out_index;
  const uint32_t* kq;
  uint32_t k_stride;
  uint32_t* done;
};

// One thread computes one candidate's exact distance in the host kernel's
// summation order, with that kernel's SIMD lanes as separate accumulators in
// registers (the warp-per-row forms, bdist / bdist_neon, reduce the same
// lanes across threads by the same tree), so a query's candidates are all
// in flight at once instead of one row per round trip.
//   NEON: 16 chains (element 16i + l into chain l; 4-blocks continue chains
//   0..3), the tree ((c0+c4)+(c8+c12))+((c1+c5)+(c9+c13)) + ... of the
//   4 / 8 / 1 / 2 butterfly, then the scalar tail fused in order.
//   AVX-512: chains A0..A31 and B0..B31 (64-blocks: 64i + l into A_l,
//   64i + 32 + l into B_l; 16-blocks into A0..A15; the masked remainder into
//   A16..), s_l = (A_l + A_l+16) + (B_l + B_l+16), then the 8 / 4 / 2 / 1
//   butterfly over s_0..s_15.
template <bool L2>
__device__ __forceinline__ float ex_term(float q, float x, float acc) {
  if (L2) {
    const float d = __fsub_rn(q, x);
    return __fmaf_rn(d, d, acc);
  }
  return __fmaf_rn(q, x, acc);
}

template <bool L2>
__device__ float exact_dist_neon(const float* __restrict__ x, const float* q, uint32_t dim) {
  const uint32_t n16 = dim / 16, n4 = (dim % 16) / 4, tail = dim % 4;
  float c[16];
#pragma unroll
  for (int l = 0; l < 16; ++l) c[l] = 0.0f;
  const float4* xv = reinterpret_cast<const float4*>(x);
  for (uint32_t i = 0; i < n16; ++i) {
    float4 v[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) v[j] = __ldg(xv + 4 * i + j);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      c[4 * j] = ex_term<L2>(q[16 * i + 4 * j], v[j].x, c[4 * j]);
      c[4 * j + 1] = ex_term<L2>(q[16 * i + 4 * j + 1], v[j].y, c[4 * j + 1]);
      c[4 * j + 2] = ex_term<L2>(q[16 * i + 4 * j + 2], v[j].z, c[4 * j + 2]);
      c[4 * j + 3] = ex_term<L2>(q[16 * i + 4 * j + 3], v[j].w, c[4 * j + 3]);
    }
  }
  for (uint32_t j = 0; j < n4; ++j) {
    const uint32_t e = 16 * n16 + 4 * j;
    const float4 v = __ldg(xv + e / 4);
    c[0] = ex_term<L2>(q[e], v.x, c[0]);
    c[1] = ex_term<L2>(q[e + 1], v.y, c[1]);
    c[2] = ex_term<L2>(q[e + 2], v.z, c[2]);
    c[3] = ex_term<L2>(q[e + 3], v.w, c[3]);
  }
  float r2[4];  // lanes 0..3 after the 4 and 8 levels
#pragma unroll
  for (int l = 0; l < 4; ++l)
    r2[l] = __fadd_rn(__fadd_rn(c[l], c[l + 4]), __fadd_rn(c[l + 8], c[l + 12]));
  float s = __fadd_rn(__fadd_rn(r2[0], r2[1]), __fadd_rn(r2[2], r2[3]));
  for (uint32_t t = 0; t < tail; ++t) {
    const uint32_t e = 16 * n16 + 4 * n4 + t;
    s = ex_term<L2>(q[e], __ldg(x + e), s);
  }
  return L2 ? s : __fsub_rn(1.0f, s);
}

template <bool L2>
__device__ float exact_dist_avx512(const float* __restrict__ x, const float* q, uint32_t dim) {
  const uint32_t nb = dim / 64, nt = (dim % 64) / 16, rem = dim % 16;
  float a[32], b[32];
#pragma unroll
  for (int l = 0; l < 32; ++l) a[l] = b[l] = 0.0f;
  const float4* xv = reinterpret_cast<const float4*>(x);
  for (uint32_t i = 0; i < nb; ++i) {
    float4 v[16];
#pragma unroll
    for (int j = 0; j < 16; ++j) v[j] = __ldg(xv + 16 * i + j);
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const uint32_t e = 64 * i + 4 * j;
      a[4 * j] = ex_term<L2>(q[e], v[j].x, a[4 * j]);
      a[4 * j + 1] = ex_term<L2>(q[e + 1], v[j].y, a[4 * j + 1]);
      a[4 * j + 2] = ex_term<L2>(q[e + 2], v[j].z, a[4 * j + 2]);
      a[4 * j + 3] = ex_term<L2>(q[e + 3], v[j].w, a[4 * j + 3]);
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const uint32_t e = 64 * i + 32 + 4 * j;
      b[4 * j] = ex_term<L2>(q[e], v[8 + j].x, b[4 * j]);
      b[4 * j + 1] = ex_term<L2>(q[e + 1], v[8 + j].y, b[4 * j + 1]);
      b[4 * j + 2] = ex_term<L2>(q[e + 2], v[8 + j].z, b[4 * j + 2]);
      b[4 * j + 3] = ex_term<L2>(q[e + 3], v[8 + j].w, b[4 * j + 3]);
    }
  }
  for (uint32_t u = 0; u < nt; ++u) {
    const uint32_t e0 = 64 * nb + 16 * u;
    float4 v[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) v[j] = __ldg(xv + e0 / 4 + j);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      a[4 * j] = ex_term<L2>(q[e0 + 4 * j], v[j].x, a[4 * j]);
      a[4 * j + 1] = ex_term<L2>(q[e0 + 4 * j + 1], v[j].y, a[4 * j + 1]);
      a[4 * j + 2] = ex_term<L2>(q[e0 + 4 * j + 2], v[j].z, a[4 * j + 2]);
      a[4 * j + 3] = ex_term<L2>(q[e0 + 4 * j + 3], v[j].w, a[4 * j + 3]);
    }
  }
  if (rem) {
    const uint32_t e0 = 64 * nb + 16 * nt;
#pragma unroll
    for (int l = 0; l < 16; ++l)
      if (static_cast<uint32_t>(l) < rem) a[16 + l] = ex_term<L2>(q[e0 + l], __ldg(x + e0 + l), a[16 + l]);
  }
  float sv[16];
#pragma unroll
  for (int l = 0; l < 16; ++l) sv[l] = __fadd_rn(__fadd_rn(a[l], a[l + 16]), __fadd_rn(b[l], b[l + 16]));
  float t8[8];
#pragma unroll
  for (int l = 0; l < 8; ++l) t8[l] = __fadd_rn(sv[l], sv[l + 8]);
  const float s = __fadd_rn(__fadd_rn(__fadd_rn(t8[0], t8[4]), __fadd_rn(t8[2], t8[6])),
                            __fadd_rn(__fadd_rn(t8[1], t8[5]), __fadd_rn(t8[3], t8[7])));
  return L2 ? s : __fsub_rn(1.0f, s);
}

// One CTA per query: the exact distances of the pool, a block bitonic sort,
// the first k written.  Queries: row q at queries + q * qstride (cosine: times
// inv[q] when inv is given).  Shared memory: the query (dim rounded up to 4)
// and p2max keys.
// After the bound pass: per query, an upper bound of the k-th smallest of
// its tile-part minima -- each minimum is a different row's score, so k rows
// score at or below it, and the bound plus the margin bounds the k-th
// distance over all rows -- published as the query's starting threshold
// (gkey).  Two 8-bit radix passes over the order-preserving keys find the
// 16-bit key prefix holding the k-th smallest; the bound is the largest key
// with that prefix.  One CTA per 32 queries, reads coalesced across queries.
constexpr int kBndThreads = 256;
__global__ void __launch_bounds__(kBndThreads) bound_select_kernel(const float* __restrict__ mins, uint32_t nq,
                                                                   uint32_t nq_pad, uint32_t m, uint32_t k,
                                                                   const float* __restrict__ qm, uint32_t* gkey) {
  __shared__ uint32_t hist[32][257];
  __shared__ uint32_t pick[32], below[32];
  const int t = threadIdx.x, j = t & 31, r0 = t >> 5;
  const uint32_t q = blockIdx.x * 32u + static_cast<uint32_t>(j);
  for (int pass = 0; pass < 2; ++pass) {
    for (int i = t; i < 32 * 257; i += kBndThreads) (&hist[0][0])[i] = 0u;
    __syncthreads();
    const uint32_t want = pass == 0 ? 0u : pick[j];
    for (uint32_t r = static_cast<uint32_t>(r0); r < m; r += kBndThreads / 32) {
      const uint32_t key = okey(__ldg(mins + static_cast<size_t>(r) * nq_pad + blockIdx.x * 32u + j));
      if (pass == 0) atomicAdd(&hist[j][key >> 24], 1u);
      else if ((key >> 24) == want) atomicAdd(&hist[j][(key >> 16) & 0xFFu], 1u);
    }
    __syncthreads();
    if (t < 32) {
      uint32_t run = pass == 0 ? 0u : below[t], b = 256u;
      for (uint32_t i = 0; i < 256u; ++i) {
        if (run + hist[t][i] >= k) {
          b = i;
          break;
        }
        run += hist[t][i];
      }
      if (pass == 0) {
        pick[t] = b;
        below[t] = run;
      } else {
        pick[t] = b == 256u ? 0xFFFFFFFFu : ((pick[t] << 24) | (b << 16) | 0xFFFFu);
      }
    }
    if (pass == 0 && t < 32 && pick[t] == 256u) pick[t] = 0xFFFFFFFFu;  // fewer than k minima: no bound
    __syncthreads();
  }
  if (t < 32 && q < nq) {
    const uint32_t bk = pick[t];
    if (bk != 0xFFFFFFFFu) {
      const float b = dist_of_key_bits(bk);
      if (isfinite(b)) gkey[q] = okey(__fadd_ru(b, qm[q]));
    }
  }
}

constexpr int kRerankThreads = 128;

template <bool L2, bool NEON>
__global__ void __launch_bounds__(kRerankThreads) rerank_kernel(
    const float* __restrict__ rows, const uint64_t* __restrict__ labels, const float* __restrict__ queries,
    uint32_t qstride, const float* __restrict__ inv, uint32_t dim, uint32_t dp, uint32_t k,
    const uint32_t* __restrict__ pool, uint32_t pool_cap, const uint32_t* __restrict__ pool_n, Rec* __restrict__ out,
    OutMap om) {
  extern __shared__ __align__(16) unsigned char smem[];
  const uint32_t dq = (dim + 3u) & ~3u;
  float* qsm = reinterpret_cast<float*>(smem);
  uint64_t* keys = reinterpret_cast<uint64_t*>(smem + ((dq * 4u + 15u) & ~15u));
  const uint32_t q = blockIdx.x;
  const int t = threadIdx.x;
  const float iv = inv ? inv[q] : 1.0f;
  for (uint32_t i = t; i < dq; i += kRerankThreads) {
    const float v = i < dim ? queries[static_cast<size_t>(q) * qstride + i] : 0.0f;
    qsm[i] = inv ? __fmul_rn(v, iv) : v;
  }
  __syncthreads();
  const uint32_t m = pool_n[q];
  const uint32_t* ids = pool + static_cast<size_t>(q) * pool_cap;
  for (uint32_t c = t; c < m; c += kRerankThreads) {
    const uint32_t r = ids[c];
    const float* x = rows + static_cast<size_t>(r) * dp;
    const float d = NEON ? exact_dist_neon<L2>(x, qsm, dim) : exact_dist_avx512<L2>(x, qsm, dim);
    keys[c] = (static_cast<uint64_t>(okey(d)) << 32) | r;
  }
  uint32_t p2 = 1;
  while (p2 < m) p2 <<= 1;
  for (uint32_t i = m + t; i < p2; i += kRerankThreads) keys[i] = ~0ull;
  __syncthreads();
  for (uint32_t kk = 2; kk <= p2; kk <<= 1) {
    for (uint32_t j = kk >> 1; j > 0; j >>= 1) {
      for (uint32_t i = t; i < p2; i += kRerankThreads) {
        const uint32_t l = i ^ j;
        if (l > i) {
          const uint64_t x0 = keys[i], x1 = keys[l];
          if ((x0 > x1) == ((i & kk) == 0)) {
            keys[i] = x1;
            keys[l] = x0;
          }
        }
      }
      __syncthreads();
    }
  }
  const uint32_t orow = om.out_index ? om.out_index[q] : q;
  const uint32_t stride = om.k_stride ? om.k_stride : k;
  const uint32_t kk_row = om.kq ? om.kq[orow] : k;
  const uint32_t mv = m < kk_row ? m : kk_row;
  Rec* row = out + static_cast<size_t>(orow) * stride;
  for (uint32_t j = t; j < stride; j += kRerankThreads) {
    Rec o;
    if (j < mv) {
      const uint64_t kv = keys[j];
      o.label = labels[static_cast<uint32_t>(kv)];
      o.dist = key_dist(kv);
    } else {
      o.label = ~0ull;
      o.dist = __int_as_float(0x7f800000);
    }
    o.zero = 0;
    row[j] = o;
  }
  if (om.done) {
    __threadfence_system();
    __syncthreads();
    if (t == 0) *reinterpret_cast<volatile uint32_t*>(om.done + orow) = 1u;
  }
}

// nq queries, one CTA each; p2max = the pool capacity rounded up to a power of two
template <bool L2>
cudaError_t launch_rerank(uint32_t nq, uint32_t p2max, bool neon, cudaStream_t st, const float* rows,
                          const uint64_t* labels, const float* queries, uint32_t qstride, const float* inv,
                          uint32_t dim, uint32_t dp, uint32_t k, const uint32_t* pool, uint32_t pool_cap,
                          const uint32_t* pool_n, Rec* out, OutMap om) {
  if (nq == 0) return cudaSuccess;
  const size_t smem = ((((dim + 3u) & ~3u) * 4u + 15u) & ~15u) + static_cast<size_t>(p2max) * 8u;
  auto go = [&](auto fn) {
    cudaError_t e = open_smem_limit(reinterpret_cast<const void*>(fn));
    if (e != cudaSuccess) return e;
    fn<<<nq, kRerankThreads, smem, st>>>(rows, labels, queries, qstride, inv, dim, dp, k, pool, pool_cap, pool_n, out,
                                         om);
    return cudaGetLastError();
  };
  return neon ? go(rerank_kernel<L2, true>) : go(rerank_kernel<L2, false>);
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }();
  return fn;
}

// K-major FP16 matrix [rows][kp] with a (64 x box_rows) box and 128-byte swizzle
bool make_map(CUtensorMap* m, const void* base, uint64_t rows, uint32_t kp, uint32_t box_rows) {
  auto fn = encode_fn();
  if (!fn) return false;
  const cuuint64_t dims[2] = {kp, rows};
  const cuuint64_t strides[1] = {static_cast<cuuint64_t>(kp) * 2};
  const cuuint32_t box[2] = {static_cast<cuuint32_t>(BK), box_rows};
  const cuuint32_t estr[2] = {1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

uint32_t round_up(uint32_t v, uint32_t m) { return (v + m - 1) / m * m; }

struct Buf {
  void* p = nullptr;
  size_t n = 0;
  cudaError_t ensure(size_t bytes) {
    if (bytes <= n) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    const cudaError_t e = cudaMalloc(&p, std::max<size_t>(bytes, 256));
    if (e == cudaSuccess) n = std::max<size_t>(bytes, 256);
    return e;
  }
  template <typename T>
  T* as() const {
    return static_cast<T*>(p);
  }
  ~Buf() {
    if (p) cudaFree(p);
  }
};

}  // namespace

// Device buffers of one scan, grown on demand and reused across calls.
struct Scratch {
  Buf qp, q16, qc, qm, qq, buf, cnt, pool, pool_n, err, tiles, gkey, mins;
};

struct Store {
  __half* x16 = nullptr;
  float* xn = nullptr;
  uint32_t n_pad = 0, kp = 0;
  DataBound db{};
  CUtensorMap map_x{};
  int sms = 0;
  std::mutex mu;  // one search() at a time uses `sc`
  Scratch sc;
};

bool supported(uint32_t dim, uint32_t k) { return dim >= 1 && dim <= kMaxDim && k >= 1 && k <= kMaxK; }

cudaError_t store_create(const Rows& r, cudaStream_t st, Store** out, std::string* err) {
  auto* s = new Store();
  s->kp = round_up(r.dim, BK);
  s->n_pad = round_up(std::max<uint32_t>(r.n, 1), BN);
  cudaError_t e = cudaSuccess;
  RowStats* dstats = nullptr;
  auto fail = [&](const char* what) {
    *err = std::string("tensor brute force: ") + what + ": " + cudaGetErrorString(e);
    if (dstats) cudaFree(dstats);
    store_free(s);
    return e;
  };
  int dev = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return fail("device");
  if ((e = cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return fail("device");
  if ((e = cudaMalloc(&s->x16, static_cast<size_t>(s->n_pad) * s->kp * 2)) != cudaSuccess) return fail("alloc");
  if ((e = cudaMalloc(&s->xn, static_cast<size_t>(s->n_pad) * 4)) != cudaSuccess) return fail("alloc");
  if ((e = cudaMalloc(&dstats, sizeof(RowStats))) != cudaSuccess) return fail("alloc");
  RowStats init{0u, 0u, 0u, 1u};
  if ((e = cudaMemcpyAsync(dstats, &init, sizeof(init), cudaMemcpyHostToDevice, st)) != cudaSuccess) return fail("copy");
  if (r.n) {
    row_stats_kernel<<<static_cast<unsigned>((static_cast<uint64_t>(r.n) * 32 + 255) / 256), 256, 0, st>>>(
        r.rows, r.n, r.dim, r.dp, dstats);
    if ((e = cudaGetLastError()) != cudaSuccess) return fail("stats kernel");
  }
  RowStats hs{};
  if ((e = cudaMemcpyAsync(&hs, dstats, sizeof(hs), cudaMemcpyDeviceToHost, st)) != cudaSuccess) return fail("copy");
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return fail("stats");
  cudaFree(dstats);
  dstats = nullptr;
  float xm, x1, x2;
  std::memcpy(&xm, &hs.max_abs_bits, 4);
  std::memcpy(&x1, &hs.max_l1_bits, 4);
  std::memcpy(&x2, &hs.max_l2_bits, 4);
  s->db.all_int = hs.all_int != 0u;
  s->db.xm = xm;
  s->db.x1 = x1;
  s->db.x2 = x2;
  s->db.sigma_x = 1.0f;
  if (!s->db.all_int && xm > 0.0f) {
    int ex;
    std::frexp(xm, &ex);
    s->db.sigma_x = std::ldexp(1.0f, 14 - ex);
  }
  encode_rows_kernel<<<static_cast<unsigned>((static_cast<uint64_t>(s->n_pad) * 32 + 255) / 256), 256, 0, st>>>(
      r.rows, r.n, s->n_pad, r.dim, r.dp, s->kp, s->db.sigma_x, r.metric == HGD_METRIC_L2 ? 1 : 0, s->x16, s->xn);
  if ((e = cudaGetLastError()) != cudaSuccess) return fail("encode kernel");
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return fail("encode");
  if (!make_map(&s->map_x, s->x16, s->n_pad, s->kp, BN)) {
    e = cudaErrorInvalidValue;
    return fail("tensor map");
  }
  *out = s;
  return cudaSuccess;
}

void store_free(Store* s) {
  if (!s) return;
  if (s->x16) cudaFree(s->x16);
  if (s->xn) cudaFree(s->xn);
  delete s;
}

// Row-tile step of the bound pass: the largest power of two that still
// samples about 96 row tiles (192 for k >= 64) and at least 4k tile-part
// minima per query.  Measured on 200k and 1M rows: 8 and 32 at k = 10, 4 and
// 8-16 at k = 100 (host calls within 5% of the best step).
uint32_t bound_step(uint32_t nbt, uint32_t k, uint32_t parts) {
  const uint32_t want = k >= 64 ? 192u : 96u;
  uint32_t step = 1;
  while (step < 1024u && nbt / (2 * step) >= want &&
         static_cast<uint64_t>(parts) * (nbt / (2 * step)) >= 4ull * k)
    step *= 2;
  return step;
}

cudaError_t open_mma_limits() {
  cudaError_t e = open_smem_limit(reinterpret_cast<const void*>(bf_mma_kernel<8>));
  return e == cudaSuccess ? open_smem_limit(reinterpret_cast<const void*>(bf_mma_kernel<16>)) : e;
}

cudaError_t launch_mma(bool wide, unsigned grid, const CUtensorMap& map_q, const CUtensorMap& map_x,
                       const MmaParams& P, cudaStream_t st) {
  if (wide) bf_mma_kernel<16><<<grid, Epi<16>::kThreads, kSmem, st>>>(map_q, map_x, P);
  else bf_mma_kernel<8><<<grid, Epi<8>::kThreads, kSmem, st>>>(map_q, map_x, P);
  return cudaGetLastError();
}

// Row splits of the scan (work items = query tiles x splits on a persistent
// grid of one CTA per SM): from the count that gives one item per SM up to
// four times it, the one with the shortest critical path, waves x (row tiles
// per split + a per-item overhead).  Every split adds its own candidates to
// the select step, so a batch of few queries takes one wave, not two.  The overhead, 64 + 2k row tiles, was
// fitted to measured 1M-row scans: every item restarts its queries'
// thresholds, and the select kernel reads every split's candidates.  Fewest
// splits on ties; the candidate buffers stay within 1 GiB.
void choose_splits(uint32_t tiles_q, uint32_t nbt, uint32_t sms, uint32_t k, uint64_t bytes_per_split,
                   uint32_t* splits_out, uint32_t* tps_out, bool seeded, uint32_t parts) {
  const uint32_t s0 = std::min<uint32_t>(std::min<uint32_t>(nbt, kSelMaxSplits / parts),
                                         std::max<uint32_t>(1, (sms + tiles_q - 1) / tiles_q));
  uint32_t s_hi = std::min<uint32_t>(std::min<uint32_t>(nbt, kSelMaxSplits / parts), 4u * s0);  // parts buffer sets per split
  while (s_hi > s0 && static_cast<uint64_t>(s_hi) * bytes_per_split > (1ull << 30)) --s_hi;
  // seeded thresholds (the bound pass) do not restart with each item
  const uint64_t overhead = seeded ? 16u : 64u + 2u * static_cast<uint64_t>(k);
  uint64_t best = ~0ull;
  for (uint32_t s = s0; s <= s_hi; ++s) {
    const uint32_t tps = (nbt + s - 1) / s;
    const uint32_t splits = (nbt + tps - 1) / tps;
    const uint64_t items = static_cast<uint64_t>(tiles_q) * splits;
    const uint64_t waves = (items + sms - 1) / sms;
    const uint64_t t = waves * (tps + overhead);
    if (t < best) {
      best = t;
      *splits_out = splits;
      *tps_out = tps;
    }
  }
}

cudaError_t search(Store* s, const Rows& r, const float* queries, const float* inv, uint32_t nq, uint32_t k,
                   const uint32_t* allow, void* out, cudaStream_t st, bool* redo, std::string* err) {
  *redo = false;
  if (nq == 0) return cudaSuccess;
  const uint32_t nq_pad = round_up(nq, BM);
  const uint32_t tiles_q = nq_pad / BM;
  const uint32_t nbt = s->n_pad / BN;
  const uint32_t cap = std::max<uint32_t>(256, round_up(2 * k + 64, 32));
  uint32_t splits = 1, tps = nbt;
  // the bound pass (the GEMM over every tstep-th row tile, keeping only each
  // tile part's smallest score per query) seeds every query's threshold
  // before the scan, for batches of many query tiles while its minima fit
  // 1 GiB (10k x 200k rows, k = 10: 2.20 -> 1.51 ms per call; 4,096 x 1M:
  // 2.49 -> 1.93 ms; for few queries a second launch costs more than it
  // saves).
  const bool wide = tiles_q >= kWideEpiTiles;
  const uint32_t parts = wide ? Epi<16>::kParts : Epi<8>::kParts;
  const uint32_t tstep = bound_step(nbt, k, parts);
  const uint32_t nbt_s = (nbt + tstep - 1) / tstep;  // row tiles the bound pass samples
  const uint64_t mins_bytes = static_cast<uint64_t>(parts) * nbt_s * nq_pad * 4;
  const bool seeded = wide && (tstep > 1 || k >= 64) && mins_bytes <= (1ull << 30);
  choose_splits(tiles_q, nbt, static_cast<uint32_t>(s->sms), k, static_cast<uint64_t>(parts) * nq_pad * cap * 8,
                &splits, &tps, seeded, parts);
  const uint32_t subs = parts * splits;  // candidate buffers per query: one per (split, tile part)
  const uint32_t pool_cap = std::min<uint32_t>(kMaxPool, round_up(std::max<uint32_t>(subs * cap, 32), 32));
  uint32_t p2max = 1;
  while (p2max < pool_cap) p2max <<= 1;

  std::lock_guard<std::mutex> lock(s->mu);
  Scratch& sc = s->sc;
  cudaError_t e = cudaSuccess;
  const char* what = "";
  do {
    what = "alloc";
    if ((e = sc.q16.ensure(static_cast<size_t>(nq_pad) * s->kp * 2)) != cudaSuccess) break;
    if ((e = sc.qc.ensure(nq_pad * 4ull)) != cudaSuccess) break;
    if ((e = sc.qm.ensure(nq_pad * 4ull)) != cudaSuccess) break;
    if ((e = sc.qq.ensure(nq_pad * 4ull)) != cudaSuccess) break;
    if ((e = sc.buf.ensure(static_cast<size_t>(subs) * nq * cap * 8)) != cudaSuccess) break;
    if ((e = sc.cnt.ensure(static_cast<size_t>(subs) * nq * 4)) != cudaSuccess) break;
    if ((e = sc.pool.ensure(static_cast<size_t>(nq) * pool_cap * 4)) != cudaSuccess) break;
    if ((e = sc.pool_n.ensure(nq * 4ull)) != cudaSuccess) break;
    if ((e = sc.err.ensure(16)) != cudaSuccess) break;
    if ((e = sc.gkey.ensure(nq * 4ull)) != cudaSuccess) break;
    if ((e = cudaMemsetAsync(sc.gkey.p, 0xFF, nq * 4ull, st)) != cudaSuccess) break;
    __half* q16 = sc.q16.as<__half>();
    float *qc = sc.qc.as<float>(), *qm = sc.qm.as<float>(), *qq = sc.qq.as<float>();
    uint64_t* buf = sc.buf.as<uint64_t>();
    uint32_t *cnt = sc.cnt.as<uint32_t>(), *pool = sc.pool.as<uint32_t>(), *pool_n = sc.pool_n.as<uint32_t>();
    uint32_t* derr = sc.err.as<uint32_t>();
    // counts of (split, query) pairs an aborted CTA never reached read as 0
    if ((e = cudaMemsetAsync(cnt, 0, static_cast<size_t>(subs) * nq * 4, st)) != cudaSuccess) break;
    if ((e = cudaMemsetAsync(derr, 0, 16, st)) != cudaSuccess) break;
    what = "query kernel";
    prep_queries_kernel<<<static_cast<unsigned>((static_cast<uint64_t>(nq_pad) * 32 + 255) / 256), 256, 0, st>>>(
        queries, inv, nq, nq_pad, r.dim, s->kp, r.metric == HGD_METRIC_L2 ? 1 : 0, s->db, q16, qc, qm, qq);
    if ((e = cudaGetLastError()) != cudaSuccess) break;
    CUtensorMap map_q;
    what = "tensor map";
    if (!make_map(&map_q, q16, nq_pad, s->kp, BM)) {
      e = cudaErrorInvalidValue;
      break;
    }
    MmaParams P{};
    P.xn = s->xn;
    P.allow = allow;
    P.qc = qc;
    P.qm = qm;
    P.buf = buf;
    P.cnt = cnt;
    P.err = derr;
    P.gkey = sc.gkey.as<uint32_t>();
    P.n = r.n;
    P.nq = nq;
    P.kchunks = s->kp / BK;
    P.cap = cap;
    P.trig = std::min<uint32_t>(cap, std::max<uint32_t>(96, round_up(2 * k + 64, 32)));
    // a small k compacts first after one appended chunk: every sub-split's
    // threshold starts at +inf, so its first rows all pass
    P.trig0 = k <= 31 ? 63u : P.trig;
    P.tstep = 1;
    P.k = k;
    P.nbt = nbt;
    P.tiles_q = tiles_q;
    P.splits = splits;
    P.tps = tps;
    P.l2 = r.metric == HGD_METRIC_L2 ? 1 : 0;
    what = "tensor kernel";
    if ((e = open_mma_limits()) != cudaSuccess) break;
    const uint32_t items = tiles_q * splits;
    const unsigned grid = std::min<uint32_t>(items, static_cast<uint32_t>(s->sms));
    if (seeded) {
      what = "alloc";
      if ((e = sc.mins.ensure(mins_bytes)) != cudaSuccess) break;
      what = "bound pass";
      MmaParams B = P;
      B.bound_pass = 1;
      B.mins = sc.mins.as<float>();
      B.nq_pad = nq_pad;
      B.tstep = tstep;
      if ((e = launch_mma(wide, grid, map_q, s->map_x, B, st)) != cudaSuccess) break;
      bound_select_kernel<<<nq_pad / 32, kBndThreads, 0, st>>>(B.mins, nq, nq_pad, parts * nbt_s, k, qm, P.gkey);
      if ((e = cudaGetLastError()) != cudaSuccess) break;
      what = "tensor kernel";
    }
    if ((e = launch_mma(wide, grid, map_q, s->map_x, P, st)) != cudaSuccess) break;
    what = "select kernel";
    select_cta_kernel<<<nq, kSelThreads, 0, st>>>(buf, cnt, qm, qq, nq, subs, cap, k, pool, pool_cap, pool_n, derr,
                                                  0, nullptr, nullptr, nullptr);
    if ((e = cudaGetLastError()) != cudaSuccess) break;
    what = "rerank kernel";
    e = r.metric == HGD_METRIC_L2
            ? launch_rerank<true>(nq, p2max, r.neon != 0, st, r.rows, r.labels, queries, r.dim, inv, r.dim, r.dp, k,
                                  pool, pool_cap, pool_n, static_cast<Rec*>(out), OutMap{nullptr, nullptr, 0, nullptr})
            : launch_rerank<false>(nq, p2max, r.neon != 0, st, r.rows, r.labels, queries, r.dim, inv, r.dim, r.dp, k,
                                   pool, pool_cap, pool_n, static_cast<Rec*>(out), OutMap{nullptr, nullptr, 0, nullptr});
    if (e != cudaSuccess) break;
    uint32_t herr[4] = {0, 0, 0, 0};
    what = "status";
    if ((e = cudaMemcpyAsync(herr, derr, 16, cudaMemcpyDeviceToHost, st)) != cudaSuccess) break;
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) break;
    if (herr[0]) {
      e = cudaErrorLaunchTimeout;
      what = "tensor pipeline wait expired";
      break;
    }
    *redo = herr[1] != 0;
  } while (false);
  if (e != cudaSuccess) *err = std::string("tensor brute force: ") + what + ": " + cudaGetErrorString(e);
  cudaStreamSynchronize(st);  // the scratch is free for the next call
  return e;
}

namespace {

// Routed queries, prepared (cosine: times 1/||q||) and zero-padded to the
// rows' padded width: qp[i] = query qlist[i].
__global__ void gather_queries_kernel(const float* __restrict__ raw, const float* __restrict__ inv,
                                      const uint32_t* __restrict__ qlist, uint32_t n_r, uint32_t dim, uint32_t pd,
                                      float* __restrict__ qp) {
  const uint64_t i = (static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= n_r) return;
  const uint32_t q = qlist[i];
  const float iv = inv ? inv[q] : 1.0f;
  for (uint32_t e = lane; e < pd; e += 32) {
    const float v = e < dim ? raw[static_cast<size_t>(q) * dim + e] : 0.0f;
    qp[i * pd + e] = inv ? __fmul_rn(v, iv) : v;
  }
}


// ---------------------------------------------------------------------------
// Routed scans over the allowed rows only
// ---------------------------------------------------------------------------
// The routed queries of a graph batch are few per filter, and their filters
// allow a small share of the rows.  The GEMM above reads every row for a tile
// of 128 queries and holds an SM's shared memory for the whole scan; this
// kernel reads only the rows a filter allows, for 8 queries at a time, with
// 16 KB of shared memory per 4 warps, so it runs beside graph walks.
//
// One warp per (tile, segment).  A tile is up to 8 consecutive routed queries
// with the same filter (the host sorts the routed queries by filter); a
// segment is a range of 32-row words.  A round turns 32 words of allow and
// alive bits into row ids (a warp scan of their counts), then scores them 16
// rows per mma.sync m16n8k16 (rows as A, the tile's queries as B, FP32
// accumulation) straight from the store's FP16 rows with 16-byte loads: lane
// (g, t) holds the elements [32t, 32t + 32) of a 128-element chunk of rows g
// and g + 8 and of query g, and uses elements 32t + 4s .. 32t + 4s + 3 at
// k-step s.  That permutes the dot product's terms, identically for A and
// B, so the score is the GEMM's s = |x|^2 + acc * qc (or acc * qc) up to the
// summation order, which the error bound already covers.
//
// Candidates go to the same per-(segment, query) buffers, with the same
// compaction and margin, as the GEMM's.  A compaction's bound is the k-th
// smallest score of a subset of the rows plus the margin, never below the
// bound over all rows, so it is safe for every segment: it is published in a
// per-query word (atomicMin on the order-preserving key) that every segment
// reads once per round.
struct SparseParams {
  const __half* x16;         // n_pad x kp store rows
  const float* xn;           // n_pad
  const __half* q16;         // nq_pad x kp prepared routed queries
  const float* qc;           // per routed query
  const float* qm;           // per routed query: selection margin
  const uint32_t* kq;        // per original query k, or null (k)
  const uint32_t* qlist;     // routed query -> original query
  const uint2* tiles;        // {first routed query, queries (1..8)}
  const uint32_t* const* allow_tab;
  const int32_t* fsel;       // per routed query
  const uint32_t* alive;     // or null
  uint64_t* buf;             // segs x nq x cap
  uint32_t* cnt;             // segs x nq
  uint32_t* gkey;            // per routed query: tightest published bound (key bits)
  uint32_t n, nq, kp, cap, k, segs, wps, words, ntiles;
  int l2;
  uint32_t sample;  // > 0: only the first `sample` (<= 16) allowed rows of each segment, every score kept
};

constexpr int kSpWarps = 4;
constexpr uint32_t kSpRound = 16;  // words per round: one per lane of the lower half
constexpr uint32_t kNoId = 0xFFFFFFFFu;

struct SparseQ {  // per tile query, warp-uniform (shared memory)
  uint32_t cnt, lim, trig, k;
  float margin;
  uint32_t over;
};

// CH = kp / 128 chunks per row.  Shared memory per warp: the round's row ids
// and the lane's B fragments (uint2 per k-step, lane-major: conflict-free).
template <int CH>
__global__ void __launch_bounds__(kSpWarps * 32, 4) sparse_scan_kernel(SparseParams P) {
  __shared__ uint32_t ids_all[kSpWarps][kSpRound * 32];
  __shared__ uint2 bfrag_all[kSpWarps][CH * 8][32];
  __shared__ SparseQ qs_all[kSpWarps][8];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t gw = blockIdx.x * kSpWarps + static_cast<uint32_t>(warp);
  const uint32_t tile = gw / P.segs, seg = gw % P.segs;
  if (tile >= P.ntiles) return;
  uint32_t* ids = ids_all[warp];
  uint2 (*bfrag)[32] = bfrag_all[warp];
  SparseQ* qs = qs_all[warp];
  const uint2 td = P.tiles[tile];
  const uint32_t q0 = td.x, nqt = td.y;
  const int g = lane >> 2, t = lane & 3;
  const uint32_t* allow = P.allow_tab[P.fsel[q0]];
  if (lane < static_cast<int>(nqt)) {
    const uint32_t q = q0 + static_cast<uint32_t>(lane);
    SparseQ z;
    z.k = P.kq ? min(P.kq[P.qlist[q]], P.k) : P.k;
    z.trig = min(P.cap, max(96u, (2u * z.k + 64u + 31u) / 32u * 32u));
    z.cnt = 0u;
    z.lim = z.trig;
    z.margin = P.qm[q];
    z.over = 0u;
    qs[lane] = z;
  }
  // query g's words [16t, 16t + 16) of each chunk (zero past the tile), as
  // the B fragments of the eight k-steps
#pragma unroll
  for (int c = 0; c < CH; ++c) {
    uint32_t w[16];
    if (static_cast<uint32_t>(g) < nqt) {
      const uint4* p = reinterpret_cast<const uint4*>(P.q16 + static_cast<size_t>(q0 + g) * P.kp + 128 * c + 32 * t);
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const uint4 u = __ldg(p + i);
        w[4 * i] = u.x;
        w[4 * i + 1] = u.y;
        w[4 * i + 2] = u.z;
        w[4 * i + 3] = u.w;
      }
    } else {
#pragma unroll
      for (int i = 0; i < 16; ++i) w[i] = 0u;
    }
#pragma unroll
    for (int st = 0; st < 8; ++st) bfrag[8 * c + st][lane] = make_uint2(w[2 * st], w[2 * st + 1]);
  }
  // this lane's two query columns 2t, 2t + 1
  const bool va = 2u * t < nqt, vb = 2u * t + 1u < nqt;
  const uint32_t qa = q0 + 2u * t, qb = qa + 1u;
  const float cqa = va ? P.qc[qa] : 0.0f, cqb = vb ? P.qc[qb] : 0.0f;
  uint32_t lka = va ? 0xFF800000u : 0u, lkb = vb ? 0xFF800000u : 0u;  // pass: key <= lk (+inf: all finite)
  __syncwarp();
  const uint32_t lt_mask = (1u << lane) - 1u;
  const uint32_t w_begin = seg * P.wps, w_end = min(P.words, w_begin + P.wps);
  for (uint32_t wb = w_begin; wb < w_end; wb += kSpRound) {
    // the tightest bound published so far
    if (va) lka = min(lka, *reinterpret_cast<volatile const uint32_t*>(P.gkey + qa));
    if (vb) lkb = min(lkb, *reinterpret_cast<volatile const uint32_t*>(P.gkey + qb));
    const uint32_t wi = wb + static_cast<uint32_t>(lane);
    uint32_t bits = 0u;
    if (lane < static_cast<int>(kSpRound) && wi < w_end) {
      bits = __ldg(allow + wi);
      if (P.alive) bits &= __ldg(P.alive + wi);
      const uint32_t r0 = wi * 32u;
      if (r0 + 32u > P.n) bits &= P.n > r0 ? ((1u << (P.n - r0)) - 1u) : 0u;  // P.n - r0 < 32 here
    }
    const uint32_t c = static_cast<uint32_t>(__popc(bits));
    uint32_t incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t u = __shfl_up_sync(kFull, incl, o);
      if (lane >= o) incl += u;
    }
    const uint32_t m_all = __shfl_sync(kFull, incl, 31);
    uint32_t pos = incl - c;
    while (bits) {
      const int b = __ffs(bits) - 1;
      bits &= bits - 1u;
      ids[pos++] = wi * 32u + static_cast<uint32_t>(b);
    }
    __syncwarp();
    const uint32_t m = P.sample ? min(m_all, P.sample) : m_all;
    for (uint32_t base = 0; base < m; base += 16u) {
      const uint32_t r0 = base + static_cast<uint32_t>(g), r1 = r0 + 8u;
      const uint32_t i0 = r0 < m ? ids[r0] : kNoId, i1 = r1 < m ? ids[r1] : kNoId;
      float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
      for (int ch = 0; ch < CH; ++ch) {
        uint32_t a[2][16];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const uint32_t r = h ? i1 : i0;
          if (r != kNoId) {
            const uint4* p = reinterpret_cast<const uint4*>(P.x16 + static_cast<size_t>(r) * P.kp + 128 * ch + 32 * t);
#pragma unroll
            for (int i = 0; i < 4; ++i) {
              const uint4 u = __ldg(p + i);
              a[h][4 * i] = u.x;
              a[h][4 * i + 1] = u.y;
              a[h][4 * i + 2] = u.z;
              a[h][4 * i + 3] = u.w;
            }
          } else {
#pragma unroll
            for (int i = 0; i < 16; ++i) a[h][i] = 0u;
          }
        }
#pragma unroll
        for (int st = 0; st < 8; ++st) {
          const uint2 b = bfrag[8 * ch + st][lane];
          sp_mma(acc, a[0][2 * st], a[1][2 * st], a[0][2 * st + 1], a[1][2 * st + 1], b.x, b.y);
        }
      }
      // acc: (row g, column 2t), (row g, 2t + 1), (row g + 8, 2t), (row g + 8, 2t + 1)
      const float x0 = (P.l2 && i0 != kNoId) ? __ldg(P.xn + i0) : 0.0f;
      const float x1 = (P.l2 && i1 != kNoId) ? __ldg(P.xn + i1) : 0.0f;
      auto score = [&](float d, float cq, float x) { return P.l2 ? __fmaf_rn(d, cq, x) : __fmul_rn(d, cq); };
      const uint32_t ka0 = okey(score(acc[0], cqa, x0)), kb0 = okey(score(acc[1], cqb, x0));
      const uint32_t ka1 = okey(score(acc[2], cqa, x1)), kb1 = okey(score(acc[3], cqb, x1));
      const bool pa0 = i0 != kNoId && ka0 <= lka, pb0 = i0 != kNoId && kb0 <= lkb;
      const bool pa1 = i1 != kNoId && ka1 <= lka, pb1 = i1 != kNoId && kb1 <= lkb;
      if (!__any_sync(kFull, pa0 || pb0 || pa1 || pb1)) continue;  // the common case once bounds settle
#pragma unroll 1
      for (int j = 0; j < 8; ++j) {
        const bool mine = t == (j >> 1);
        const bool p0 = mine && ((j & 1) ? pb0 : pa0), p1 = mine && ((j & 1) ? pb1 : pa1);
        const uint32_t bal0 = __ballot_sync(kFull, p0), bal1 = __ballot_sync(kFull, p1);
        if ((bal0 | bal1) == 0u) continue;
        const uint32_t q = q0 + static_cast<uint32_t>(j);
        uint64_t* bufp = P.buf + (static_cast<size_t>(seg) * P.nq + q) * P.cap;
        const uint32_t c0 = qs[j].cnt;
        const uint32_t n0 = static_cast<uint32_t>(__popc(bal0));
        if (p0) bufp[c0 + __popc(bal0 & lt_mask)] = (static_cast<uint64_t>((j & 1) ? kb0 : ka0) << 32) | i0;
        if (p1) bufp[c0 + n0 + __popc(bal1 & lt_mask)] = (static_cast<uint64_t>((j & 1) ? kb1 : ka1) << 32) | i1;
        const uint32_t c1 = c0 + n0 + static_cast<uint32_t>(__popc(bal1));
        __syncwarp();
        if (c1 + 16u <= qs[j].lim) {
          __syncwarp();
          if (lane == 0) qs[j].cnt = c1;
          __syncwarp();
          continue;
        }
        // room for the next group: compact, publish the bound
        float thr;
        const uint32_t kept = warp_compact(bufp, c1, qs[j].k, qs[j].margin, lane, &thr);
        const uint32_t key = okey(thr);
        const bool over = kept + 16u > P.cap;  // the margin keeps too many rows: stop adding (lenient)
        if (mine) {
          if (j & 1) lkb = over ? 0u : min(lkb, key);
          else lka = over ? 0u : min(lka, key);
        }
        __syncwarp();
        if (lane == 0) {
          qs[j].cnt = kept;
          qs[j].lim = min(P.cap, max(qs[j].trig, kept + 64u));
          qs[j].over = over ? 1u : 0u;
          if (!over) atomicMin(P.gkey + q, key);
        }
        __syncwarp();
      }
    }
    __syncwarp();
    if (P.sample && m > 0) break;  // the segment's sample is taken
  }
  __syncwarp();
  if (lane < static_cast<int>(nqt)) P.cnt[static_cast<size_t>(seg) * P.nq + q0 + lane] = qs[lane].cnt;
}

}  // namespace


Scratch* scratch_new() { return new Scratch(); }
void scratch_free(Scratch* s) { delete s; }

namespace {

// Tiles of the sparse scan: runs of routed queries with the same filter
// (fsel sorted), cut into pieces of at most 8.
std::vector<uint2> routed_tiles(const int32_t* fsel, uint32_t n_r) {
  std::vector<uint2> tiles;
  for (uint32_t i = 0; i < n_r;) {
    uint32_t j = i + 1;
    while (j < n_r && j - i < 8 && fsel[j] == fsel[i]) ++j;
    tiles.push_back(make_uint2(i, j - i));
    i = j;
  }
  return tiles;
}

cudaError_t routed_sparse(Store* s, const Rows& r, const RoutedArgs& a, Scratch* sc, cudaStream_t st,
                          const std::vector<uint2>& tiles, const char** what) {
  const uint32_t n_r = a.n_r;
  const uint32_t k = a.k_stride;
  const uint32_t nq_pad = round_up(n_r, BM);
  const uint32_t T = static_cast<uint32_t>(tiles.size());
  const uint32_t words = (r.n + 31) / 32;
  // segments: about 128 allowed rows (8 groups) per warp for the largest
  // filter, at most 8192 warps in all and kSelMaxSplits per tile.  The
  // sample pass (16 rows of every segment) bounds each query's scores
  // before the scan, so the number of segments does not add candidates.
  uint64_t max_ones = 1;
  for (const uint2& t : tiles) max_ones = std::max<uint64_t>(max_ones, a.h_ones[a.h_fsel[t.x]]);
  uint32_t segs = static_cast<uint32_t>(std::min<uint64_t>(kSelMaxSplits, (max_ones + 127) / 128));
  segs = std::max<uint32_t>(1, std::min<uint32_t>(segs, std::max<uint32_t>(1, 8192 / T)));
  const uint32_t wps = round_up((words + segs - 1) / segs, kSpRound);
  segs = std::max<uint32_t>(1, (words + wps - 1) / wps);
  const uint32_t cap = std::max<uint32_t>(256, round_up(2 * k + 64, 32));
  const uint32_t pool_cap = std::min<uint32_t>(kMaxPool, round_up(2 * cap, 32));
  uint32_t p2max = 1;
  while (p2max < pool_cap) p2max <<= 1;
  cudaError_t e = cudaSuccess;
  *what = "alloc";
  if ((e = sc->qp.ensure(static_cast<size_t>(n_r) * r.dp * 4)) != cudaSuccess) return e;
  if ((e = sc->q16.ensure(static_cast<size_t>(nq_pad) * s->kp * 2)) != cudaSuccess) return e;
  if ((e = sc->qc.ensure(nq_pad * 4ull)) != cudaSuccess) return e;
  if ((e = sc->qm.ensure(nq_pad * 4ull)) != cudaSuccess) return e;
  if ((e = sc->qq.ensure(nq_pad * 4ull)) != cudaSuccess) return e;
  if ((e = sc->buf.ensure(static_cast<size_t>(segs) * n_r * cap * 8)) != cudaSuccess) return e;
  if ((e = sc->cnt.ensure(static_cast<size_t>(segs) * n_r * 4)) != cudaSuccess) return e;
  if ((e = sc->pool.ensure(static_cast<size_t>(n_r) * pool_cap * 4)) != cudaSuccess) return e;
  if ((e = sc->pool_n.ensure(n_r * 4ull)) != cudaSuccess) return e;
  if ((e = sc->err.ensure(16)) != cudaSuccess) return e;
  if ((e = sc->tiles.ensure(T * sizeof(uint2))) != cudaSuccess) return e;
  if ((e = sc->gkey.ensure(n_r * 4ull)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(sc->err.p, 0, 16, st)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(sc->gkey.p, 0xFF, n_r * 4ull, st)) != cudaSuccess) return e;
  if ((e = cudaMemcpyAsync(sc->tiles.p, tiles.data(), T * sizeof(uint2), cudaMemcpyHostToDevice, st)) != cudaSuccess)
    return e;
  *what = "gather kernel";
  gather_queries_kernel<<<static_cast<unsigned>((static_cast<uint64_t>(n_r) * 32 + 255) / 256), 256, 0, st>>>(
      a.queries, a.inv, a.qlist, n_r, a.dim, r.dp, sc->qp.as<float>());
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  *what = "query kernel";
  prep_queries_kernel<<<static_cast<unsigned>((static_cast<uint64_t>(nq_pad) * 32 + 255) / 256), 256, 0, st>>>(
      sc->qp.as<float>(), nullptr, n_r, nq_pad, r.dim, s->kp, r.metric == HGD_METRIC_L2 ? 1 : 0, s->db,
      sc->q16.as<__half>(), sc->qc.as<float>(), sc->qm.as<float>(), sc->qq.as<float>());
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  SparseParams P{};
  P.x16 = s->x16;
  P.xn = s->xn;
  P.q16 = sc->q16.as<__half>();
  P.qc = sc->qc.as<float>();
  P.qm = sc->qm.as<float>();
  P.kq = a.kq;
  P.qlist = a.qlist;
  P.tiles = sc->tiles.as<uint2>();
  P.allow_tab = a.allow_tab;
  P.fsel = a.fsel;
  P.alive = a.alive;
  P.buf = sc->buf.as<uint64_t>();
  P.cnt = sc->cnt.as<uint32_t>();
  P.gkey = sc->gkey.as<uint32_t>();
  P.n = r.n;
  P.nq = n_r;
  P.kp = s->kp;
  P.cap = cap;
  P.k = k;
  P.segs = segs;
  P.wps = wps;
  P.words = words;
  P.ntiles = T;
  P.l2 = r.metric == HGD_METRIC_L2 ? 1 : 0;
  const unsigned grid = static_cast<unsigned>((static_cast<uint64_t>(T) * segs + kSpWarps - 1) / kSpWarps);
  auto scan = [&](uint32_t sample) {
    P.sample = sample;
    switch (s->kp / 128) {
      case 1: sparse_scan_kernel<1><<<grid, kSpWarps * 32, 0, st>>>(P); break;
      case 2: sparse_scan_kernel<2><<<grid, kSpWarps * 32, 0, st>>>(P); break;
      case 3: sparse_scan_kernel<3><<<grid, kSpWarps * 32, 0, st>>>(P); break;
      case 4: sparse_scan_kernel<4><<<grid, kSpWarps * 32, 0, st>>>(P); break;
      default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
  };
  // the sample (at most 4096 rows per query, held in the bound kernel's
  // registers) and its bound (the k-th smallest sampled score + the margin
  // bounds the k-th smallest of all rows from above), then the scan
  *what = "sample scan kernel";
  if ((e = scan(std::max<uint32_t>(1, std::min<uint32_t>(16, 4096 / segs)))) != cudaSuccess) return e;
  *what = "bound kernel";
  select_cta_kernel<<<n_r, kSelThreads, 0, st>>>(sc->buf.as<uint64_t>(), sc->cnt.as<uint32_t>(), sc->qm.as<float>(),
                                                 sc->qq.as<float>(), n_r, segs, cap, k, nullptr, 0, nullptr,
                                                 sc->err.as<uint32_t>(), 1, a.kq, a.qlist, sc->gkey.as<uint32_t>());
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  *what = "sparse scan kernel";
  if ((e = scan(0)) != cudaSuccess) return e;
  *what = "select kernel";
  select_cta_kernel<<<n_r, kSelThreads, 0, st>>>(sc->buf.as<uint64_t>(), sc->cnt.as<uint32_t>(), sc->qm.as<float>(),
                                                 sc->qq.as<float>(), n_r, segs, cap, k, sc->pool.as<uint32_t>(),
                                                 pool_cap, sc->pool_n.as<uint32_t>(), sc->err.as<uint32_t>(), 1, a.kq,
                                                 a.qlist, nullptr);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  *what = "rerank kernel";
  const OutMap om{a.qlist, a.kq, a.k_stride, a.done};
  return r.metric == HGD_METRIC_L2
             ? launch_rerank<true>(n_r, p2max, r.neon != 0, st, r.rows, r.labels, sc->qp.as<float>(), r.dp, nullptr,
                                   r.dim, r.dp, k, sc->pool.as<uint32_t>(), pool_cap, sc->pool_n.as<uint32_t>(),
                                   static_cast<Rec*>(a.out), om)
             : launch_rerank<false>(n_r, p2max, r.neon != 0, st, r.rows, r.labels, sc->qp.as<float>(), r.dp, nullptr,
                                    r.dim, r.dp, k, sc->pool.as<uint32_t>(), pool_cap, sc->pool_n.as<uint32_t>(),
                                    static_cast<Rec*>(a.out), om);
}

// Whether the allowed-rows scan reads fewer bytes than the GEMM (within 2x:
// it also runs beside the walks, the GEMM holds whole SMs).
bool routed_prefers_rows(uint32_t kp, const int32_t* fsel, uint32_t n_r, const uint64_t* ones, uint32_t n) {
  if (kp % 128 != 0 || kp > 512 || n_r == 0) return false;
  const std::vector<uint2> tiles = routed_tiles(fsel, n_r);
  uint64_t rows = 0;
  for (const uint2& t : tiles) rows += ones[fsel[t.x]];
  const uint64_t tiles_q = (n_r + BM - 1) / BM;
  return rows <= 2ull * tiles_q * n;
}

}  // namespace

cudaError_t search_routed(Store* s, const Rows& r, const RoutedArgs& a, Scratch* sc, cudaStream_t st,
                          std::string* err) {
  if (a.n_r == 0) return cudaSuccess;
  const char* what = "alloc";
  bool rows_only = a.h_fsel != nullptr && a.h_ones != nullptr && s->kp % 128 == 0 && s->kp <= 512;
  if (rows_only && a.mode == HGD_SCAN_AUTO) rows_only = routed_prefers_rows(s->kp, a.h_fsel, a.n_r, a.h_ones, r.n);
  if (rows_only && a.mode == HGD_SCAN_EVERY_ROW) rows_only = false;
  if (rows_only) {
    const cudaError_t e = routed_sparse(s, r, a, sc, st, routed_tiles(a.h_fsel, a.n_r), &what);
    if (e != cudaSuccess && err) *err = std::string("routed scan: ") + what + ": " + cudaGetErrorString(e);
    return e;
  }
  const uint32_t n_r = a.n_r;
  const uint32_t k = a.k_stride;
  const uint32_t nq_pad = round_up(n_r, BM);
  const uint32_t tiles_q = nq_pad / BM;
  const uint32_t nbt = s->n_pad / BN;
  const uint32_t cap = std::max<uint32_t>(256, round_up(2 * k + 64, 32));
  uint32_t splits = 1, tps = nbt;
  // the bound pass (the GEMM over every tstep-th row tile, keeping only each
  // tile part's smallest score per query) seeds every query's threshold
  // before the scan, for batches of many query tiles while its minima fit
  // 1 GiB (10k x 200k rows, k = 10: 2.20 -> 1.51 ms per call; 4,096 x 1M:
  // 2.49 -> 1.93 ms; for few queries a second launch costs more than it
  // saves).
  const bool wide = tiles_q >= kWideEpiTiles;
  const uint32_t parts = wide ? Epi<16>::kParts : Epi<8>::kParts;
  const uint32_t tstep = bound_step(nbt, k, parts);
  const uint32_t nbt_s = (nbt + tstep - 1) / tstep;  // row tiles the bound pass samples
  const uint64_t mins_bytes = static_cast<uint64_t>(parts) * nbt_s * nq_pad * 4;
  const bool seeded = wide && (tstep > 1 || k >= 64) && mins_bytes <= (1ull << 30);
  choose_splits(tiles_q, nbt, static_cast<uint32_t>(s->sms), k, static_cast<uint64_t>(parts) * nq_pad * cap * 8,
                &splits, &tps, seeded, parts);
  const uint32_t subs = parts * splits;  // candidate buffers per query: one per (split, tile part)
  const uint32_t pool_cap = std::min<uint32_t>(kMaxPool, round_up(std::max<uint32_t>(subs * cap, 32), 32));
  uint32_t p2max = 1;
  while (p2max < pool_cap) p2max <<= 1;
  cudaError_t e = cudaSuccess;
  do {
    if ((e = sc->qp.ensure(static_cast<size_t>(n_r) * r.dp * 4)) != cudaSuccess) break;
    if ((e = sc->q16.ensure(static_cast<size_t>(nq_pad) * s->kp * 2)) != cudaSuccess) break;
    if ((e = sc->qc.ensure(nq_pad * 4ull)) != cudaSuccess) break;
    if ((e = sc->qm.ensure(nq_pad * 4ull)) != cudaSuccess) break;
    if ((e = sc->qq.ensure(nq_pad * 4ull)) != cudaSuccess) break;
    if ((e = sc->buf.ensure(static_cast<size_t>(subs) * n_r * cap * 8)) != cudaSuccess) break;
    if ((e = sc->cnt.ensure(static_cast<size_t>(subs) * n_r * 4)) != cudaSuccess) break;
    if ((e = sc->pool.ensure(static_cast<size_t>(n_r) * pool_cap * 4)) != cudaSuccess) break;
    if ((e = sc->pool_n.ensure(n_r * 4ull)) != cudaSuccess) break;
    if ((e = sc->err.ensure(16)) != cudaSuccess) break;
    if ((e = sc->gkey.ensure(n_r * 4ull)) != cudaSuccess) break;
    if ((e = cudaMemsetAsync(sc->gkey.p, 0xFF, n_r * 4ull, st)) != cudaSuccess) break;
    if ((e = cudaMemsetAsync(sc->cnt.p, 0, static_cast<size_t>(subs) * n_r * 4, st)) != cudaSuccess) break;
    if ((e = cudaMemsetAsync(sc->err.p, 0, 16, st)) != cudaSuccess) break;
    what = "gather kernel";
    gather_queries_kernel<<<static_cast<unsigned>((static_cast<uint64_t>(n_r) * 32 + 255) / 256), 256, 0, st>>>(
        a.queries, a.inv, a.qlist, n_r, a.dim, r.dp, sc->qp.as<float>());
    if ((e = cudaGetLastError()) != cudaSuccess) break;
    what = "query kernel";
    prep_queries_kernel<<<static_cast<unsigned>((static_cast<uint64_t>(nq_pad) * 32 + 255) / 256), 256, 0, st>>>(
        sc->qp.as<float>(), nullptr, n_r, nq_pad, r.dim, s->kp, r.metric == HGD_METRIC_L2 ? 1 : 0, s->db,
        sc->q16.as<__half>(), sc->qc.as<float>(), sc->qm.as<float>(), sc->qq.as<float>());
    if ((e = cudaGetLastError()) != cudaSuccess) break;
    CUtensorMap map_q;
    what = "tensor map";
    if (!make_map(&map_q, sc->q16.p, nq_pad, s->kp, BM)) {
      e = cudaErrorInvalidValue;
      break;
    }
    MmaParams P{};
    P.xn = s->xn;
    P.qc = sc->qc.as<float>();
    P.qm = sc->qm.as<float>();
    P.buf = sc->buf.as<uint64_t>();
    P.cnt = sc->cnt.as<uint32_t>();
    P.err = sc->err.as<uint32_t>();
    P.allow_tab = a.allow_tab;
    P.fsel = a.fsel;
    P.alive = a.alive;
    P.gkey = sc->gkey.as<uint32_t>();
    P.n = r.n;
    P.nq = n_r;
    P.kchunks = s->kp / BK;
    P.cap = cap;
    P.trig = std::min<uint32_t>(cap, std::max<uint32_t>(96, round_up(2 * k + 64, 32)));
    // a small k compacts first after one appended chunk: every sub-split's
    // threshold starts at +inf, so its first rows all pass
    P.trig0 = k <= 31 ? 63u : P.trig;
    P.tstep = 1;
    P.k = k;
    P.nbt = nbt;
    P.tiles_q = tiles_q;
    P.splits = splits;
    P.tps = tps;
    P.l2 = r.metric == HGD_METRIC_L2 ? 1 : 0;
    P.lenient = 1;
    what = "tensor kernel";
    if ((e = open_mma_limits()) != cudaSuccess) break;
    const unsigned grid = std::min<uint32_t>(tiles_q * splits, static_cast<uint32_t>(s->sms));
    if (seeded) {
      // k_stride bounds every routed query's k: its bound is safe for each
      what = "alloc";
      if ((e = sc->mins.ensure(mins_bytes)) != cudaSuccess) break;
      what = "bound pass";
      MmaParams B = P;
      B.bound_pass = 1;
      B.mins = sc->mins.as<float>();
      B.nq_pad = nq_pad;
      B.tstep = tstep;
      if ((e = launch_mma(wide, grid, map_q, s->map_x, B, st)) != cudaSuccess) break;
      bound_select_kernel<<<nq_pad / 32, kBndThreads, 0, st>>>(B.mins, n_r, nq_pad, parts * nbt_s, k, P.qm, P.gkey);
      if ((e = cudaGetLastError()) != cudaSuccess) break;
      what = "tensor kernel";
    }
    if ((e = launch_mma(wide, grid, map_q, s->map_x, P, st)) != cudaSuccess) break;
    what = "select kernel";
    select_cta_kernel<<<n_r, kSelThreads, 0, st>>>(sc->buf.as<uint64_t>(), sc->cnt.as<uint32_t>(), sc->qm.as<float>(),
                                                   sc->qq.as<float>(), n_r, subs, cap, k, sc->pool.as<uint32_t>(),
                                                   pool_cap, sc->pool_n.as<uint32_t>(), sc->err.as<uint32_t>(), 1, a.kq,
                                                   a.qlist, nullptr);
    if ((e = cudaGetLastError()) != cudaSuccess) break;
    what = "rerank kernel";
    const OutMap om{a.qlist, a.kq, a.k_stride, a.done};
    e = r.metric == HGD_METRIC_L2
            ? launch_rerank<true>(n_r, p2max, r.neon != 0, st, r.rows, r.labels, sc->qp.as<float>(), r.dp, nullptr,
                                  r.dim, r.dp, k, sc->pool.as<uint32_t>(), pool_cap, sc->pool_n.as<uint32_t>(),
                                  static_cast<Rec*>(a.out), om)
            : launch_rerank<false>(n_r, p2max, r.neon != 0, st, r.rows, r.labels, sc->qp.as<float>(), r.dp, nullptr,
                                   r.dim, r.dp, k, sc->pool.as<uint32_t>(), pool_cap, sc->pool_n.as<uint32_t>(),
                                   static_cast<Rec*>(a.out), om);
  } while (false);
  if (e != cudaSuccess && err) *err = std::string("tensor scan: ") + what + ": " + cudaGetErrorString(e);
  return e;
}

}  // namespace hg::bfm
