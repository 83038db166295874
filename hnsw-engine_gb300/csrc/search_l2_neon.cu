// search_l2_neon.cu -- instantiations of the query kernel for the squared-L2 metric,
// distances in the NEON kernel's summation order (indexes loaded on Arm
// hosts, where the reference dispatches to its NEON kernels).
#include "search_kernel.cuh"

namespace hg {

cudaError_t launch_search_l2_neon(const SearchParams& P, const float* inv, int blocks, int wpb, cudaStream_t st) {
  const uint32_t pd = P.pd;
  HG_SEARCH_DISPATCH_NEON(sk::launch_t, true, P, inv, blocks, wpb, st)
  return cudaErrorInvalidValue;
}

int occupancy_l2_neon(uint32_t pd, int wpb, size_t smem) {
  HG_SEARCH_DISPATCH_NEON(sk::occupancy_t, true, wpb, smem)
  return 0;
}

}  // namespace hg
