// search_beam.cu -- instantiations of the beam walk (one warp per query,
// several lists per step, tensor-core distances) for the compressed copies
// of rows of 128 elements: both metric families, with and without filters
// or deletes.
#include "search_beam.cuh"

namespace hg {

namespace {
template <int PREC, bool L2>
cudaError_t launch_p(const SearchParams& P, const float* inv, int blocks, int wpb, bool filt, cudaStream_t st) {
  return filt ? sk::beam_launch_t<PREC, L2, true>(P, inv, blocks, wpb, st)
              : sk::beam_launch_t<PREC, L2, false>(P, inv, blocks, wpb, st);
}
template <int PREC, bool L2>
int occ_p(int wpb, size_t smem, bool filt) {
  return filt ? sk::beam_occupancy_t<PREC, L2, true>(wpb, smem) : sk::beam_occupancy_t<PREC, L2, false>(wpb, smem);
}
}  // namespace

cudaError_t launch_search_beam(const SearchParams& P, const float* inv, int blocks, int wpb, bool filt,
                               cudaStream_t st) {
  if (P.pdc != 128) return cudaErrorInvalidValue;
  const bool fp8 = P.vscale != nullptr;
  if (P.metric == 0)
    return fp8 ? launch_p<2, true>(P, inv, blocks, wpb, filt, st) : launch_p<1, true>(P, inv, blocks, wpb, filt, st);
  return fp8 ? launch_p<2, false>(P, inv, blocks, wpb, filt, st) : launch_p<1, false>(P, inv, blocks, wpb, filt, st);
}

int occupancy_beam(int metric, int prec, int wpb, size_t smem, bool filt) {
  if (metric == 0) return prec == 2 ? occ_p<2, true>(wpb, smem, filt) : occ_p<1, true>(wpb, smem, filt);
  return prec == 2 ? occ_p<2, false>(wpb, smem, filt) : occ_p<1, false>(wpb, smem, filt);
}

}  // namespace hg
