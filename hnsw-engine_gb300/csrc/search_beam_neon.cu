// search_beam_neon.cu -- the beam walk with its exact rerank in the NEON
// kernel's summation order (indexes on Arm hosts).
#include "search_beam.cuh"

namespace hg {

cudaError_t launch_search_beam_neon(const SearchParams& P, const float* inv, int blocks, int wpb, bool filt,
                                    cudaStream_t st) {
  return sk::beam_launch<1>(P, inv, blocks, wpb, filt, st);
}

int occupancy_beam_neon(int metric, int prec, int wpb, size_t smem, bool filt) {
  return sk::beam_occupancy<1>(metric, prec, wpb, smem, filt);
}

}  // namespace hg
