// rerank.cu -- the row encoders that build the FP16 / FP8-E4M3 copies of the
// vectors walked by the compressed-precision traversal (whose exact FP32
// rerank is fused into the traversal kernel).
#include <cuda_fp16.h>
#include <cuda_fp8.h>

#include "search_kernel.cuh"

namespace hg {

namespace {

// one warp per row: FP16 copy, zero padded to pdc
__global__ void encode_f16_kernel(const float* __restrict__ vecs, uint32_t n, uint32_t pd, uint32_t pdc,
                                  __half* __restrict__ out) {
  const uint64_t row = (static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  for (uint32_t i = lane; i < pdc; i += 32)
    out[row * pdc + i] = __float2half_rn(i < pd ? vecs[row * pd + i] : 0.0f);
}

// one warp per row: scale = max|x| / 448 (the largest finite E4M3 value),
// e = E4M3(x / scale) with saturation; zero rows keep scale 1
__global__ void encode_f8_kernel(const float* __restrict__ vecs, uint32_t n, uint32_t pd, uint32_t pdc,
                                 uint8_t* __restrict__ out, float* __restrict__ scale) {
  const uint64_t row = (static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  float mx = 0.0f;
  for (uint32_t i = lane; i < pd; i += 32) mx = fmaxf(mx, fabsf(vecs[row * pd + i]));
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xFFFFFFFFu, mx, o));
  const float s = mx > 0.0f ? mx / 448.0f : 1.0f;
  for (uint32_t i = lane; i < pdc; i += 32) {
    const float x = i < pd ? vecs[row * pd + i] / s : 0.0f;
    out[row * pdc + i] = __nv_cvt_float_to_fp8(x, __NV_SATFINITE, __NV_E4M3);
  }
  if (lane == 0) scale[row] = s;
}

}  // namespace

cudaError_t launch_encode(const float* vecs, uint32_t n, uint32_t pd, uint32_t pdc, int prec, void* out,
                          float* scale, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  const unsigned blocks = static_cast<unsigned>((static_cast<uint64_t>(n) * 32 + 255) / 256);
  if (prec == 1) encode_f16_kernel<<<blocks, 256, 0, st>>>(vecs, n, pd, pdc, static_cast<__half*>(out));
  else encode_f8_kernel<<<blocks, 256, 0, st>>>(vecs, n, pd, pdc, static_cast<uint8_t*>(out), scale);
  return cudaGetLastError();
}

}  // namespace hg
