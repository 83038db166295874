// bf_common.cuh -- the brute-force distance orders shared by the CUDA-core
// scan and the tensor-core path's rerank (reference src/brute_force.cpp:34-69
// sums over `dim`, not the padded width, with the host's kernel: the AVX-512
// one of src/kernels_avx512.cpp on x86-64, the NEON one of
// src/kernels_neon.cpp on Arm).
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

// The shape of one order over dim.  AVX-512: nb 64-blocks, nt 16-blocks, a
// masked remainder of rem.  NEON: n16 16-blocks, n4 4-blocks, tail scalars.
struct BfOrder {
  int nb, nt, rem;
  int n16, n4, tail;
  bool neon;
};

__host__ __device__ inline BfOrder bf_order(uint32_t dim, bool neon) {
  BfOrder o{};
  o.neon = neon;
  o.nb = static_cast<int>(dim / 64);
  o.nt = static_cast<int>((dim % 64) / 16);
  o.rem = static_cast<int>(dim % 16);
  o.n16 = static_cast<int>(dim / 16);
  o.n4 = static_cast<int>((dim % 16) / 4);
  o.tail = static_cast<int>(dim % 4);
  return o;
}

// register slots one lane needs for a row of dim elements in the order
__host__ __device__ inline int bf_slots(uint32_t dim, bool neon) {
  const BfOrder o = bf_order(dim, neon);
  return neon ? o.n16 + o.n4 + o.tail : 2 * o.nb + o.nt + 1;
}

// Element of slot i on this lane (-1: none).
// AVX-512: A chain 64i+lane (i<nb); B chain 64i+32+lane; 16-blocks (lanes<16)
// 64nb+16u+lane; masked remainder (lanes>=16) 64nb+16nt+(lane-16) < dim.
// NEON: 16-block chains 16i+lane (lanes<16); 4-blocks into acc0, 16n16+4j+lane
// (lanes<4); the scalar tail on lane 0.
__device__ __forceinline__ int bslot(const BfOrder& o, int i, int lane) {
  if (o.neon) {
    if (i < o.n16) return lane < 16 ? 16 * i + lane : -1;
    const int j = i - o.n16;
    if (j < o.n4) return lane < 4 ? 16 * o.n16 + 4 * j + lane : -1;
    const int t = j - o.n4;
    if (t < o.tail) return lane == 0 ? 16 * o.n16 + 4 * o.n4 + t : -1;
    return -1;
  }
  const int nb = o.nb, nt = o.nt, rem = o.rem;
  if (i < nb) return 64 * i + lane;
  if (i < 2 * nb) return 64 * (i - nb) + 32 + lane;
  const int u = i - 2 * nb;
  if (u < nt) return lane < 16 ? 64 * nb + 16 * u + lane : -1;
  if (u == nt && lane >= 16 && lane - 16 < rem) return 64 * nb + 16 * nt + (lane - 16);
  return -1;
}

// NEON order: chains c = 4a + b on lanes 0..15 (4-blocks continue acc0 on
// lanes 0..3), (acc0 + acc1) + (acc2 + acc3) and vaddvq_f32 by a 4 / 8 / 1 / 2
// butterfly, then the scalar tail fused on lane 0 (as the reference's
// compiler contracts it), broadcast.
template <int S, bool L2>
__device__ __forceinline__ float bdist_neon(const float (&x)[S], const float (&q)[S], const BfOrder& o, int lane) {
  float acc = 0.0f;
#pragma unroll
  for (int i = 0; i < S; ++i) {
    const bool live = (i < o.n16 && lane < 16) || (i >= o.n16 && i < o.n16 + o.n4 && lane < 4);
    if (!live) continue;
    if (L2) {
      const float d = __fsub_rn(q[i], x[i]);
      acc = __fmaf_rn(d, d, acc);
    } else {
      acc = __fmaf_rn(q[i], x[i], acc);
    }
  }
  acc = __fadd_rn(acc, __shfl_xor_sync(kFull, acc, 4));
  acc = __fadd_rn(acc, __shfl_xor_sync(kFull, acc, 8));
  acc = __fadd_rn(acc, __shfl_xor_sync(kFull, acc, 1));
  acc = __fadd_rn(acc, __shfl_xor_sync(kFull, acc, 2));
#pragma unroll
  for (int i = 0; i < S; ++i) {
    if (i < o.n16 + o.n4 || i >= o.n16 + o.n4 + o.tail || lane != 0) continue;
    if (L2) {
      const float d = __fsub_rn(q[i], x[i]);
      acc = __fmaf_rn(d, d, acc);
    } else {
      acc = __fmaf_rn(q[i], x[i], acc);
    }
  }
  const float s = __shfl_sync(kFull, acc, 0);
  return L2 ? s : __fsub_rn(1.0f, s);
}

template <int S, bool L2>
__device__ __forceinline__ float bdist(const float (&x)[S], const float (&q)[S], const BfOrder& o, int lane) {
  if (o.neon) return bdist_neon<S, L2>(x, q, o, lane);
  const int nb = o.nb, nt = o.nt, rem = o.rem;
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
