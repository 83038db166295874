// search_approx.cu -- the query kernels on compressed rows (FP16 or per-row
// scaled FP8 E4M3, FP32 accumulation) for padded row lengths 128 / 256 /
// 512 / 1024, both metric families: one warp per query, and (rows of 128)
// four warps per query.  Both end with the fused exact FP32 rerank; the row
// encoders live in rerank.cu.
#include "search_kernel.cuh"
#include "search_wide.cuh"

namespace hg {

cudaError_t launch_search_approx(const SearchParams& P, const float* inv, int blocks, int wpb, cudaStream_t st) {
  const uint32_t pdc = P.pdc;
  const int prec = static_cast<int>(P.vscale != nullptr) + 1;  // 1 fp16, 2 fp8
  if (P.metric == 0) {
    if (prec == 1) { HG_SEARCH_APPROX_DISPATCH(sk::launch_t, 1, true, P, inv, blocks, wpb, st) }
    else { HG_SEARCH_APPROX_DISPATCH(sk::launch_t, 2, true, P, inv, blocks, wpb, st) }
  } else {
    if (prec == 1) { HG_SEARCH_APPROX_DISPATCH(sk::launch_t, 1, false, P, inv, blocks, wpb, st) }
    else { HG_SEARCH_APPROX_DISPATCH(sk::launch_t, 2, false, P, inv, blocks, wpb, st) }
  }
  return cudaErrorInvalidValue;
}

int occupancy_approx(uint32_t pdc, int metric, int prec, int wpb, size_t smem) {
  if (metric == 0) {
    if (prec == 1) { HG_SEARCH_APPROX_DISPATCH(sk::occupancy_t, 1, true, wpb, smem) }
    else { HG_SEARCH_APPROX_DISPATCH(sk::occupancy_t, 2, true, wpb, smem) }
  } else {
    if (prec == 1) { HG_SEARCH_APPROX_DISPATCH(sk::occupancy_t, 1, false, wpb, smem) }
    else { HG_SEARCH_APPROX_DISPATCH(sk::occupancy_t, 2, false, wpb, smem) }
  }
  return 0;
}

// Several warps per query (one CTA of four): the compressed layout of rows
// of 128 elements only (dim <= 128), ids below 2^24, lists of at most 32.
cudaError_t launch_search_wide(const SearchParams& P, const float* inv, int blocks, cudaStream_t st) {
  if (P.pdc != 128) return cudaErrorInvalidValue;
  const int prec = static_cast<int>(P.vscale != nullptr) + 1;
  if (P.metric == 0)
    return prec == 1 ? sk::wide_launch_t<sk::ApproxDist<4, 16, 1>, true>(P, inv, blocks, st)
                     : sk::wide_launch_t<sk::ApproxDist<4, 16, 2>, true>(P, inv, blocks, st);
  return prec == 1 ? sk::wide_launch_t<sk::ApproxDist<4, 16, 1>, false>(P, inv, blocks, st)
                   : sk::wide_launch_t<sk::ApproxDist<4, 16, 2>, false>(P, inv, blocks, st);
}

int occupancy_wide(int metric, int prec, uint32_t R) {
  const size_t smem = sk::wide_smem_bytes(R);
  if (metric == 0)
    return prec == 1 ? sk::wide_occupancy_t<sk::ApproxDist<4, 16, 1>, true>(smem)
                     : sk::wide_occupancy_t<sk::ApproxDist<4, 16, 2>, true>(smem);
  return prec == 1 ? sk::wide_occupancy_t<sk::ApproxDist<4, 16, 1>, false>(smem)
                   : sk::wide_occupancy_t<sk::ApproxDist<4, 16, 2>, false>(smem);
}

}  // namespace hg
