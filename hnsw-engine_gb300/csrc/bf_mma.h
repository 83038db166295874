// bf_mma.h -- tensor-core brute force (tcgen05 / TMEM / TMA) behind
// hgd_bruteforce: candidate selection by an FP16 GEMM with a proven error
// margin, then the exact distances of the survivors in the reference order.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>

namespace hg::bfm {

struct Store;  // FP16 K-major copy of the rows, squared norms, bound constants, TMA map

struct Rows {
  const float* rows;       // n x dp float32 (device), sorted by label, zero tail
  const uint64_t* labels;  // n (device), sorted
  uint32_t n, dim, dp;
  int metric;              // HGD_METRIC_*
  int neon;                // 1: exact distances in the NEON kernel's order, 0: the AVX-512 kernel's
};

// Whether the tensor path handles this shape (dim <= 1024, k <= 256).
bool supported(uint32_t dim, uint32_t k);

// Build the FP16 copy (once per store).  Synchronous.
cudaError_t store_create(const Rows& r, cudaStream_t st, Store** out, std::string* err);
void store_free(Store* s);

// Exact k-NN of nq device queries (raw, nq x dim); `inv` = per-query 1/||q||
// for cosine (else null), `allow` = bits over sorted rows or null.  Writes
// nq x k records to `out` (device).  On return *redo is true when some query
// could not be settled by the margin test (too many near-ties): the caller
// then answers the batch with the CUDA-core scan.  Synchronises `st`.
cudaError_t search(Store* s, const Rows& r, const float* queries, const float* inv, uint32_t nq, uint32_t k,
                   const uint32_t* allow, void* out, cudaStream_t st, bool* redo, std::string* err);

// Queries of a graph batch routed to an exact scan (the compressed-precision
// forms' answer to restrictive filters): each routed query is scanned over
// the rows its filter allows (id-space bits, 32 per word) that are alive, and
// its row of `out` (original index) is written with the first min(m, k)
// results in the graph's distance order, then its done flag.  Enqueues only.
struct RoutedArgs {
  const float* queries;              // device, nq x dim raw queries of the batch
  const float* inv;                  // device, per query 1/||q|| (cosine) or null
  const uint32_t* qlist;             // device, n_r original query indices
  const int32_t* fsel;               // device, n_r filter indices into allow_tab
  const uint32_t* const* allow_tab;  // device table of id-space bitsets
  const uint32_t* alive;             // device tombstone bits (1 = alive) or null
  uint32_t n_r, dim, k_stride;
  const uint32_t* kq;                // device per original query k, or null (k_stride)
  void* out;                         // device records, original query rows of k_stride
  uint32_t* done;                    // device per original query done flags or null
  // Host copies for the choice of scan: per routed query its filter index
  // (sorted, so queries of one filter are consecutive) and per filter the
  // number of rows it allows.  Without them the GEMM over every row runs.
  const int32_t* h_fsel;
  const uint64_t* h_ones;
  int mode;                          // HGD_SCAN_*: which scan (auto: fewer bytes)
};
struct Scratch;
Scratch* scratch_new();
void scratch_free(Scratch* s);
cudaError_t search_routed(Store* s, const Rows& r, const RoutedArgs& a, Scratch* sc, cudaStream_t st,
                          std::string* err);

}  // namespace hg::bfm
