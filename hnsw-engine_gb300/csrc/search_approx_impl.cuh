// search_approx_impl.cuh -- launch helpers of the compressed-precision walks
// (one warp per query, and four warps per query for rows of 128), templated
// on the summation order ORD of their exact FP32 rerank (0 AVX-512, 1 NEON);
// search_approx.cu and search_approx_neon.cu instantiate one order each.
#pragma once

#include "search_kernel.cuh"
#include "search_wide.cuh"

namespace hg {
namespace sk {

template <int ORD>
cudaError_t approx_launch(const SearchParams& P, const float* inv, int blocks, int wpb, cudaStream_t st) {
  const uint32_t pdc = P.pdc;
  const int prec = static_cast<int>(P.vscale != nullptr) + 1;  // 1 fp16, 2 fp8
  if (P.metric == 0) {
    if (prec == 1) { HG_SEARCH_APPROX_DISPATCH(sk::launch_t, 1, true, ORD, P, inv, blocks, wpb, st) }
    else { HG_SEARCH_APPROX_DISPATCH(sk::launch_t, 2, true, ORD, P, inv, blocks, wpb, st) }
  } else {
    if (prec == 1) { HG_SEARCH_APPROX_DISPATCH(sk::launch_t, 1, false, ORD, P, inv, blocks, wpb, st) }
    else { HG_SEARCH_APPROX_DISPATCH(sk::launch_t, 2, false, ORD, P, inv, blocks, wpb, st) }
  }
  return cudaErrorInvalidValue;
}

template <int ORD>
int approx_occupancy(uint32_t pdc, int metric, int prec, int wpb, size_t smem) {
  if (metric == 0) {
    if (prec == 1) { HG_SEARCH_APPROX_DISPATCH(sk::occupancy_t, 1, true, ORD, wpb, smem) }
    else { HG_SEARCH_APPROX_DISPATCH(sk::occupancy_t, 2, true, ORD, wpb, smem) }
  } else {
    if (prec == 1) { HG_SEARCH_APPROX_DISPATCH(sk::occupancy_t, 1, false, ORD, wpb, smem) }
    else { HG_SEARCH_APPROX_DISPATCH(sk::occupancy_t, 2, false, ORD, wpb, smem) }
  }
  return 0;
}

// Several warps per query (one CTA of four): the compressed layout of rows
// of 128 elements only (dim <= 128), ids below 2^24, lists of at most 32.
template <int ORD>
cudaError_t wide_launch(const SearchParams& P, const float* inv, int blocks, cudaStream_t st) {
  if (P.pdc != 128) return cudaErrorInvalidValue;
  const int prec = static_cast<int>(P.vscale != nullptr) + 1;
  if (P.metric == 0)
    return prec == 1 ? wide_launch_t<ApproxDist<4, 16, 1, ORD>, true>(P, inv, blocks, st)
                     : wide_launch_t<ApproxDist<4, 16, 2, ORD>, true>(P, inv, blocks, st);
  return prec == 1 ? wide_launch_t<ApproxDist<4, 16, 1, ORD>, false>(P, inv, blocks, st)
                   : wide_launch_t<ApproxDist<4, 16, 2, ORD>, false>(P, inv, blocks, st);
}

template <int ORD>
int wide_occupancy(int metric, int prec, uint32_t R) {
  const size_t smem = wide_smem_bytes(R);
  if (metric == 0)
    return prec == 1 ? wide_occupancy_t<ApproxDist<4, 16, 1, ORD>, true>(smem)
                     : wide_occupancy_t<ApproxDist<4, 16, 2, ORD>, true>(smem);
  return prec == 1 ? wide_occupancy_t<ApproxDist<4, 16, 1, ORD>, false>(smem)
                   : wide_occupancy_t<ApproxDist<4, 16, 2, ORD>, false>(smem);
}

}  // namespace sk
}  // namespace hg
