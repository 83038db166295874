// bf_common.cuh -- the brute-force distance order shared by the CUDA-core
// scan and the tensor-core path (reference src/brute_force.cpp:34-69 with the
// AVX-512 kernel of src/kernels_avx512.cpp over `dim`, not the padded width).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace hg::bf {

constexpr unsigned kFull = 0xFFFFFFFFu;


__device__ __forceinline__ uint32_t okey(float d) {
  d = __fadd_rn(d, 0.0f);
  const uint32_t u = __float_as_uint(d);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float key_dist(uint64_t key) {
  const uint32_t k = static_cast<uint32_t>(key >> 32);
  const uint32_t u = (k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k;
  return __uint_as_float(u);
}

// lane slots: A chain 64i+lane (i<nb); B chain 64i+32+lane; 16-blocks (lanes<16)
// 64nb+16u+lane; masked remainder (lanes>=16) 64nb+16nt+(lane-16) < dim.
__device__ __forceinline__ int bslot(int i, int nb, int nt, int rem, int lane) {
  if (i < nb) return 64 * i + lane;
  if (i < 2 * nb) return 64 * (i - nb) + 32 + lane;
  const int u = i - 2 * nb;
  if (u < nt) return lane < 16 ? 64 * nb + 16 * u + lane : -1;
  if (u == nt && lane >= 16 && lane - 16 < rem) return 64 * nb + 16 * nt + (lane - 16);
  return -1;
}

template <int S, bool L2>
__device__ __forceinline__ float bdist(const float (&x)[S], const float (&q)[S], int nb, int nt, int rem, int lane) {
  float a = 0.0f, b = 0.0f;
#pragma unroll
  for (int i = 0; i < S; ++i) {
    const bool chainA = i < nb || (i >= 2 * nb && i < 2 * nb + nt) || (i == 2 * nb + nt && rem > 0);
    const bool chainB = i >= nb && i < 2 * nb;
    if (!chainA && !chainB) continue;
    const int u = i - 2 * nb;
    // 16-blocks touch lanes < 16 only, the masked block lanes >= 16 only
    const bool live = chainB || i < nb || (u < nt ? lane < 16 : lane >= 16);
    if (!live) continue;
    float t;
    if (L2) {
      const float d = __fsub_rn(q[i], x[i]);
      t = __fmaf_rn(d, d, chainA ? a : b);
    } else {
      t = __fmaf_rn(q[i], x[i], chainA ? a : b);
    }
    if (chainA) a = t;
    else b = t;
  }
  const float xa = __fadd_rn(a, __shfl_xor_sync(kFull, a, 16));
  const float xb = __fadd_rn(b, __shfl_xor_sync(kFull, b, 16));
  float s = __fadd_rn(xa, xb);
  s = __fadd_rn(s, __shfl_xor_sync(kFull, s, 8));
  s = __fadd_rn(s, __shfl_xor_sync(kFull, s, 4));
  s = __fadd_rn(s, __shfl_xor_sync(kFull, s, 2));
  s = __fadd_rn(s, __shfl_xor_sync(kFull, s, 1));
  return L2 ? s : __fsub_rn(1.0f, s);
}

struct Rec {
  uint64_t label;
  float dist;
  uint32_t zero;
};

// Warp bitonic sort of keys[0..p2) ascending (p2 a power of two).
__device__ __forceinline__ void warp_sort(uint64_t* keys, int p2, int lane) {
  for (int kk = 2; kk <= p2; kk <<= 1) {
    for (int j = kk >> 1; j > 0; j >>= 1) {
      for (int i = lane; i < p2; i += 32) {
        const int l = i ^ j;
        if (l > i) {
          const uint64_t a = keys[i], b = keys[l];
          const bool up = (i & kk) == 0;
          if ((a > b) == up) {
            keys[i] = b;
            keys[l] = a;
          }
        }
      }
      __syncwarp();
    }
  }
}

}  // namespace hg::bf
