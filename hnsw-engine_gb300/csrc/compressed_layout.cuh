// compressed_layout.cuh -- element order of the FP16 / FP8-E4M3 row copies.
//
// The compressed copies are walked by tensor-core distance code (mma.sync
// m16n8k16, rows as the A operand) and by CUDA-core code (ApproxDist).  A
// row is stored in chunks of 128 elements; inside a chunk, the elements one
// thread of an MMA quad needs for its A fragments are contiguous, and one
// 16-byte load of each of the quad's four threads covers a contiguous
// 64 bytes of the row.
//
// The A fragment of m16n8k16 gives thread t (t = lane & 3) of row group g,
// at k-step s (16 dims each), the pairs (16s + 2t, +1) and (16s + 2t + 8, +9).
// Listed in that order over s = 0..7, a thread's 32 dims of a chunk form its
// "stream" e = 0..31:
//     logical(t, e) = 16 (e >> 2) + 2t + 8 ((e >> 1) & 1) + (e & 1)
// Register j of the thread (a half2) holds stream elements 2j, 2j + 1, so
// registers 2s and 2s + 1 are the fragment's a0/a2 (or a1/a3) at k-step s.
// Storage inside the chunk:
//     FP16: pos = (e >> 3) * 32 + 8 t + (e & 7)    (16 B = 8 halves)
//     FP8:  pos = (e >> 4) * 64 + 16 t + (e & 15)  (16 B = 16 bytes)
// The permutation only reorders the terms of a dot product, which the
// compressed traversal sums in any order; the exact FP32 rerank reads the
// unpermuted FP32 rows.
#pragma once

#include <cstdint>

namespace hg {

__host__ __device__ inline uint32_t stream_logical(uint32_t t, uint32_t e) {
  return 16u * (e >> 2) + 2u * t + 8u * ((e >> 1) & 1u) + (e & 1u);
}

// storage position (elements) of logical dim k; prec 1 = FP16, 2 = FP8
__host__ __device__ inline uint32_t cl_pos(uint32_t k, int prec) {
  const uint32_t c = k >> 7, r = k & 127u;
  const uint32_t s = r >> 4, u = r & 15u;
  const uint32_t t = (u & 7u) >> 1;
  const uint32_t e = 4u * s + ((u >> 3) << 1) + (u & 1u);
  const uint32_t p = prec == 1 ? (e >> 3) * 32u + 8u * t + (e & 7u) : (e >> 4) * 64u + 16u * t + (e & 15u);
  return (c << 7) + p;
}

// logical dim stored at position p (inverse of cl_pos)
__host__ __device__ inline uint32_t cl_logical(uint32_t p, int prec) {
  const uint32_t c = p >> 7, r = p & 127u;
  uint32_t t, e;
  if (prec == 1) {
    t = (r & 31u) >> 3;
    e = ((r >> 5) << 3) + (r & 7u);
  } else {
    t = (r & 63u) >> 4;
    e = ((r >> 6) << 4) + (r & 15u);
  }
  return (c << 7) + stream_logical(t, e);
}

}  // namespace hg
