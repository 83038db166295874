// search_l2.cu -- instantiations of the query kernel for the squared-L2 metric.
#include "search_kernel.cuh"

namespace hg {

cudaError_t launch_search_l2(const SearchParams& P, const float* inv, int blocks, int wpb, cudaStream_t st) {
  const uint32_t pd = P.pd;
  HG_SEARCH_DISPATCH(sk::launch_t, true, P, inv, blocks, wpb, st)
  return cudaErrorInvalidValue;
}

int occupancy_l2(uint32_t pd, int wpb, size_t smem) {
  HG_SEARCH_DISPATCH(sk::occupancy_t, true, wpb, smem)
  return 0;
}

}  // namespace hg
