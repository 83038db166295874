// search_approx.cu -- the query kernels on compressed rows (FP16 or per-row
// scaled FP8 E4M3, FP32 accumulation) for padded row lengths 128 / 256 /
// 512 / 1024, both metric families: one warp per query, and (rows of 128)
// four warps per query.  Both end with the fused exact FP32 rerank; this
// unit holds the AVX-512 rerank order and dispatches the NEON one to
// search_approx_neon.cu.  The row encoders live in rerank.cu.
#include "search_approx_impl.cuh"

namespace hg {

cudaError_t launch_search_approx_neon(const SearchParams& P, const float* inv, int blocks, int wpb, cudaStream_t st);
int occupancy_approx_neon(uint32_t pdc, int metric, int prec, int wpb, size_t smem);
cudaError_t launch_search_wide_neon(const SearchParams& P, const float* inv, int blocks, cudaStream_t st);
int occupancy_wide_neon(int metric, int prec, uint32_t R);

cudaError_t launch_search_approx(const SearchParams& P, const float* inv, int blocks, int wpb, cudaStream_t st) {
  return P.order == 1 ? launch_search_approx_neon(P, inv, blocks, wpb, st) : sk::approx_launch<0>(P, inv, blocks, wpb, st);
}

int occupancy_approx(uint32_t pdc, int metric, int prec, int order, int wpb, size_t smem) {
  return order == 1 ? occupancy_approx_neon(pdc, metric, prec, wpb, smem)
                    : sk::approx_occupancy<0>(pdc, metric, prec, wpb, smem);
}

cudaError_t launch_search_wide(const SearchParams& P, const float* inv, int blocks, cudaStream_t st) {
  return P.order == 1 ? launch_search_wide_neon(P, inv, blocks, st) : sk::wide_launch<0>(P, inv, blocks, st);
}

int occupancy_wide(int metric, int prec, int order, uint32_t R) {
  return order == 1 ? occupancy_wide_neon(metric, prec, R) : sk::wide_occupancy<0>(metric, prec, R);
}

}  // namespace hg
