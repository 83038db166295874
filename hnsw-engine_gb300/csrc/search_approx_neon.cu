// search_approx_neon.cu -- the compressed-precision walks whose exact FP32
// rerank uses the NEON kernel's summation order (indexes on Arm hosts).
#include "search_approx_impl.cuh"

namespace hg {

cudaError_t launch_search_approx_neon(const SearchParams& P, const float* inv, int blocks, int wpb, cudaStream_t st) {
  return sk::approx_launch<1>(P, inv, blocks, wpb, st);
}

int occupancy_approx_neon(uint32_t pdc, int metric, int prec, int wpb, size_t smem) {
  return sk::approx_occupancy<1>(pdc, metric, prec, wpb, smem);
}

cudaError_t launch_search_wide_neon(const SearchParams& P, const float* inv, int blocks, cudaStream_t st) {
  return sk::wide_launch<1>(P, inv, blocks, st);
}

int occupancy_wide_neon(int metric, int prec, uint32_t R) { return sk::wide_occupancy<1>(metric, prec, R); }

}  // namespace hg
