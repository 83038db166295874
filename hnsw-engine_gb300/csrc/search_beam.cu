// search_beam.cu -- instantiations of the beam walk (one warp per query,
// several lists per step, tensor-core distances) for the compressed copies
// of rows of 128 elements: both metric families, with and without filters
// or deletes, exact rerank in the AVX-512 order; the NEON order's
// instantiations are in search_beam_neon.cu.
#include "search_beam.cuh"

namespace hg {

cudaError_t launch_search_beam_neon(const SearchParams& P, const float* inv, int blocks, int wpb, bool filt,
                                    cudaStream_t st);
int occupancy_beam_neon(int metric, int prec, int wpb, size_t smem, bool filt);

cudaError_t launch_search_beam(const SearchParams& P, const float* inv, int blocks, int wpb, bool filt,
                               cudaStream_t st) {
  return P.order == 1 ? launch_search_beam_neon(P, inv, blocks, wpb, filt, st)
                      : sk::beam_launch<0>(P, inv, blocks, wpb, filt, st);
}

int occupancy_beam(int metric, int prec, int order, int wpb, size_t smem, bool filt) {
  return order == 1 ? occupancy_beam_neon(metric, prec, wpb, smem, filt)
                    : sk::beam_occupancy<0>(metric, prec, wpb, smem, filt);
}

}  // namespace hg
