// rerank.cu -- the row encoders that build the FP16 / FP8-E4M3 copies of the
// vectors walked by the compressed-precision traversal (whose exact FP32
// rerank is fused into the traversal kernels).
#include <cuda_fp16.h>
#include <cuda_fp8.h>

#include "compressed_layout.cuh"
#include "search_kernel.cuh"

namespace hg {

namespace {

// One warp per row.  Both copies store the row in the tensor-core order of
// compressed_layout.cuh (chunks of 128 elements, zero padded to pdc) and
// write aux[row] = {s, s^2 |x'|^2}: the row's scale (1 for FP16) and the
// squared norm of the stored values, for the L2 distance from a dot product.

// FP16 (round to nearest)
__global__ void encode_f16_kernel(const float* __restrict__ vecs, uint32_t n, uint32_t pd, uint32_t pdc,
                                  __half* __restrict__ out, float2* __restrict__ aux) {
  const uint64_t row = (static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  double nrm = 0.0;
  for (uint32_t i = lane; i < pdc; i += 32) {
    const __half h = __float2half_rn(i < pd ? vecs[row * pd + i] : 0.0f);
    out[row * pdc + cl_pos(i, 1)] = h;
    const double x = static_cast<double>(__half2float(h));
    nrm += x * x;
  }
  for (int o = 16; o > 0; o >>= 1) nrm += __shfl_xor_sync(0xFFFFFFFFu, nrm, o);
  if (lane == 0) aux[row] = make_float2(1.0f, static_cast<float>(nrm));
}

// FP8 E4M3: scale = max|x| / 448 (the largest finite E4M3 value),
// e = E4M3(x / scale) with saturation; zero rows keep scale 1
__global__ void encode_f8_kernel(const float* __restrict__ vecs, uint32_t n, uint32_t pd, uint32_t pdc,
                                 uint8_t* __restrict__ out, float* __restrict__ scale, float2* __restrict__ aux) {
  const uint64_t row = (static_cast<uint64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  float mx = 0.0f;
  for (uint32_t i = lane; i < pd; i += 32) mx = fmaxf(mx, fabsf(vecs[row * pd + i]));
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xFFFFFFFFu, mx, o));
  const float s = mx > 0.0f ? mx / 448.0f : 1.0f;
  double nrm = 0.0;
  for (uint32_t i = lane; i < pdc; i += 32) {
    const float x = i < pd ? vecs[row * pd + i] / s : 0.0f;
    const __nv_fp8_storage_t e = __nv_cvt_float_to_fp8(x, __NV_SATFINITE, __NV_E4M3);
    out[row * pdc + cl_pos(i, 2)] = e;
    const __half_raw hr = __nv_cvt_fp8_to_halfraw(e, __NV_E4M3);
    const double v = static_cast<double>(__half2float(__half(hr)));
    nrm += v * v;
  }
  for (int o = 16; o > 0; o >>= 1) nrm += __shfl_xor_sync(0xFFFFFFFFu, nrm, o);
  if (lane == 0) {
    scale[row] = s;
    aux[row] = make_float2(s, static_cast<float>(static_cast<double>(s) * s * nrm));
  }
}

}  // namespace

cudaError_t launch_encode(const float* vecs, uint32_t n, uint32_t pd, uint32_t pdc, int prec, void* out,
                          float* scale, float* aux, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  const unsigned blocks = static_cast<unsigned>((static_cast<uint64_t>(n) * 32 + 255) / 256);
  float2* a2 = reinterpret_cast<float2*>(aux);
  if (prec == 1) encode_f16_kernel<<<blocks, 256, 0, st>>>(vecs, n, pd, pdc, static_cast<__half*>(out), a2);
  else encode_f8_kernel<<<blocks, 256, 0, st>>>(vecs, n, pd, pdc, static_cast<uint8_t*>(out), scale, a2);
  return cudaGetLastError();
}

}  // namespace hg
