// search_aux.cu -- small kernels around the query kernel (cosine query
// norms, filter translation), the launch dispatch on metric, and the static
// scratch of the allocation-free entry point.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "search_common.cuh"

namespace hg {

cudaError_t launch_search_l2(const SearchParams& P, const float* inv, int blocks, int wpb, cudaStream_t st);
cudaError_t launch_search_dot(const SearchParams& P, const float* inv, int blocks, int wpb, cudaStream_t st);
int occupancy_l2(uint32_t pd, int wpb, size_t smem);
int occupancy_dot(uint32_t pd, int wpb, size_t smem);
cudaError_t launch_search_l2_neon(const SearchParams& P, const float* inv, int blocks, int wpb, cudaStream_t st);
cudaError_t launch_search_dot_neon(const SearchParams& P, const float* inv, int blocks, int wpb, cudaStream_t st);
int occupancy_l2_neon(uint32_t pd, int wpb, size_t smem);
int occupancy_dot_neon(uint32_t pd, int wpb, size_t smem);

namespace {

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

// Layer 0 from the file's layout (per node: count, then M0 ids) into rows of
// l0s ids padded with kNoId; the count is clamped to M0 (the host validates
// it before the graph is used).  Grid-stride over all (node, slot) pairs.
__global__ void relayout_l0_kernel(const uint32_t* __restrict__ raw, uint64_t n, uint32_t M0, uint32_t* __restrict__ l0,
                                   uint32_t l0s) {
  const uint64_t total = n * l0s;
  for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    const uint64_t node = i / l0s;
    const uint32_t j = static_cast<uint32_t>(i - node * l0s);
    const uint32_t* src = raw + node * (1ull + M0);
    const uint32_t cnt = min(__ldg(src), M0);
    l0[i] = j < cnt ? __ldg(src + 1 + j) : hg::kNoId;
  }
}

// Whether some layer-0 list (M0 <= 32) holds an id twice: one warp per list,
// one id per lane, __match_any_sync over the lanes (idle lanes hold values
// no id takes: ids are below 2^32 - 64).
__global__ void l0_dup_kernel(const uint32_t* __restrict__ raw, uint64_t n, uint32_t M0, uint32_t* __restrict__ flag) {
  const int lane = threadIdx.x & 31;
  const uint64_t warps = static_cast<uint64_t>(gridDim.x) * (blockDim.x >> 5);
  for (uint64_t node = (blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x) >> 5; node < n; node += warps) {
    const uint32_t* src = raw + node * (1ull + M0);
    const uint32_t cnt = min(__ldg(src), M0);
    const uint32_t id = static_cast<uint32_t>(lane) < cnt ? __ldg(src + 1 + lane) : 0xFFFFFFFFu - lane;
    const uint32_t same = __match_any_sync(0xFFFFFFFFu, id);
    if (__any_sync(0xFFFFFFFFu, __popc(same) > 1) && lane == 0) atomicOr(flag, 1u);
  }
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

// Sort queries into ef buckets: bucket b holds the queries whose effective
// ef (per-query or batch ef, 0 -> default, at least k) is <= hi[b].
__global__ void bucket_kernel(const uint32_t* __restrict__ efq, const uint32_t* __restrict__ kq, uint32_t nq,
                              uint32_t ef_all, uint32_t ef_default, uint32_t k_all, BucketSpec spec,
                              uint32_t* __restrict__ counts, uint32_t* __restrict__ lists,
                              const uint8_t* __restrict__ skip) {
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq) return;
  if (skip && skip[q]) return;  // answered by the exact scan
  const uint32_t k = kq ? kq[q] : k_all;
  uint32_t ef = efq ? efq[q] : ef_all;
  if (ef == 0) ef = ef_default;
  if (ef < k) ef = k;
  uint32_t b = 0;
  while (b + 1 < spec.n && ef > spec.hi[b]) ++b;
  const uint32_t pos = atomicAdd(counts + b, 1u);
  lists[static_cast<size_t>(b) * nq + pos] = q;
}

}  // namespace

cudaError_t launch_bucket(const uint32_t* efq, const uint32_t* kq, uint32_t nq, uint32_t ef_all, uint32_t ef_default,
                          uint32_t k_all, const BucketSpec& spec, uint32_t* counts, uint32_t* lists,
                          cudaStream_t st, const uint8_t* skip) {
  if (nq == 0) return cudaSuccess;
  bucket_kernel<<<(nq + 255) / 256, 256, 0, st>>>(efq, kq, nq, ef_all, ef_default, k_all, spec, counts, lists,
                                                  skip);
  return cudaGetLastError();
}

// Query slots per lane for padded dim pd (AVX-512 layout).
int slots_for(uint32_t pd) { return 2 * static_cast<int>(pd / 64) + static_cast<int>((pd % 64) / 16); }

cudaError_t launch_inv_norm(const float* qs, uint32_t nq, uint32_t dim, float* out, cudaStream_t st) {
  if (nq == 0) return cudaSuccess;
  inv_norm_kernel<<<(nq + 127) / 128, 128, 0, st>>>(qs, nq, dim, out);
  return cudaGetLastError();
}

cudaError_t launch_translate_filter(const uint64_t* label_words, uint64_t num_bits, const uint64_t* labels, uint32_t n,
                                    uint32_t* out, cudaStream_t st) {
  const uint32_t out_words = (n + 31) / 32 + 1;
  translate_filter_kernel<<<(out_words + 255) / 256, 256, 0, st>>>(label_words, num_bits, labels, n, out, out_words);
  return cudaGetLastError();
}

cudaError_t launch_relayout_l0(const uint32_t* raw, uint64_t n, uint32_t M0, uint32_t* l0, uint32_t l0s, uint32_t* dup,
                               cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  const uint64_t total = n * l0s;
  const unsigned blocks = static_cast<unsigned>(std::min<uint64_t>((total + 255) / 256, 152ull * 64));
  relayout_l0_kernel<<<blocks, 256, 0, st>>>(raw, n, M0, l0, l0s);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess || !dup) return e;
  const unsigned wblocks = static_cast<unsigned>(std::min<uint64_t>((n + 7) / 8, 152ull * 64));
  l0_dup_kernel<<<wblocks, 256, 0, st>>>(raw, n, M0, dup);
  return cudaGetLastError();
}

// Returns cudaErrorInvalidValue for a padded dimension beyond the register layouts.
cudaError_t launch_search(const SearchParams& P, const float* inv, int blocks, int warps_per_block,
                          cudaStream_t st) {
  if (P.order == 1)
    return P.metric == 0 ? launch_search_l2_neon(P, inv, blocks, warps_per_block, st)
                         : launch_search_dot_neon(P, inv, blocks, warps_per_block, st);
  return P.metric == 0 ? launch_search_l2(P, inv, blocks, warps_per_block, st)
                       : launch_search_dot(P, inv, blocks, warps_per_block, st);
}

// Resident blocks per SM of the search kernel for this shape (0 on error).
int search_occupancy(uint32_t pd, int metric, int order, int warps_per_block, uint32_t H, uint32_t R, uint32_t C) {
  const size_t smem = static_cast<size_t>(warps_per_block) * warp_smem_bytes(H, R, C);
  if (order == 1)
    return metric == 0 ? occupancy_l2_neon(pd, warps_per_block, smem) : occupancy_dot_neon(pd, warps_per_block, smem);
  return metric == 0 ? occupancy_l2(pd, warps_per_block, smem) : occupancy_dot(pd, warps_per_block, smem);
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
// A fixed 48 warps walk every batch, whatever the GPU: the per-warp scratch
// below is sized for them, so a batch runs at a fraction of the allocating
// path's throughput (which fills every SM).
constexpr int kNaWarpsPerBlock = 4;
constexpr int kNaBlocks = 12;
constexpr uint64_t kNaSlots = static_cast<uint64_t>(kNaWarpsPerBlock) * kNaBlocks;
// spill keys per warp; a query that needs more goes to the rerun pass, which
// one warp runs, so such queries are finished one after another
constexpr uint64_t kNaPoolCap = 2048;
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
// device (host code cannot use the symbol itself as a device pointer) and
// kept for the process: after a device reset the kept address would be
// stale, so a reset after the first call is not supported.
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
  // The kernel raises ctr[4] for a query whose ef or k exceeds the launch's
  // capacity.  The host checks (one ef and k per batch, R >= max(ef, k))
  // make that impossible here, so the flag is not read back; a change that
  // allowed per-query ef or k would have to read it.
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
  B.rerun = 1;
  return launch_search(B, inv, 1, 1, st);
}

}  // namespace hg
