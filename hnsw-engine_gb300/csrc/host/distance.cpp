// distance.cpp -- host distance kernels (used by the CPU graph builder) and
// the metric / ISA registry of include/hnsw/metric.hpp.
//
// Each kernel reproduces one of the reference's summation orders in portable
// C++ (explicit fmaf, no contraction: built with -ffp-contract=off), so a
// graph built here is byte-identical to one the reference builds on a host
// with that ISA:
//   scalar  sequential, separately rounded     src/kernels_scalar.cpp:9-22
//   AVX2    4x8 lanes over 32-blocks, hsum256  src/kernels_avx2.cpp:11-69
//   AVX-512 4x16 lanes over 64-blocks, masked  src/kernels_avx512.cpp:10-58
//           tail into acc1, GCC reduce_add order
//   NEON    4x4 lanes over 16-blocks, vaddvq   src/kernels_neon.cpp:10-54
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>

#include "hnsw/filter.hpp"
#include "hnsw/metric.hpp"

namespace hnsw {

Metric parse_metric(std::string_view name) {
  if (name == "l2" || name == "L2" || name == "euclidean") return Metric::L2;
  if (name == "ip" || name == "inner_product" || name == "dot") return Metric::InnerProduct;
  if (name == "cosine" || name == "angular") return Metric::Cosine;
  throw std::invalid_argument("unknown metric '" + std::string(name) + "' (expected l2, ip or cosine)");
}

std::string_view metric_name(Metric m) noexcept {
  switch (m) {
    case Metric::L2: return "l2";
    case Metric::InnerProduct: return "ip";
    case Metric::Cosine: return "cosine";
  }
  return "unknown";
}

namespace simd {
namespace {

template <bool L2>
inline float term(float x, float y, float acc) {
  if constexpr (L2) {
    const float d = x - y;
    return std::fmaf(d, d, acc);
  } else {
    return std::fmaf(x, y, acc);
  }
}

template <bool L2>
float k_scalar(const float* a, const float* b, std::size_t n) noexcept {
  float s = 0.0f;
  for (std::size_t i = 0; i < n; ++i) {
    if constexpr (L2) {
      const float d = a[i] - b[i];
      const float p = d * d;
      s = s + p;
    } else {
      const float p = a[i] * b[i];
      s = s + p;
    }
  }
  return s;
}

template <bool L2>
float k_avx2(const float* a, const float* b, std::size_t n) noexcept {
  float acc[4][8] = {};
  std::size_t i = 0;
  for (; i + 32 <= n; i += 32)
    for (int j = 0; j < 4; ++j)
      for (int l = 0; l < 8; ++l) acc[j][l] = term<L2>(a[i + 8 * j + l], b[i + 8 * j + l], acc[j][l]);
  for (; i + 8 <= n; i += 8)
    for (int l = 0; l < 8; ++l) acc[0][l] = term<L2>(a[i + l], b[i + l], acc[0][l]);
  float v[8];
  for (int l = 0; l < 8; ++l) v[l] = (acc[0][l] + acc[1][l]) + (acc[2][l] + acc[3][l]);
  float s = ((v[0] + v[4]) + (v[2] + v[6])) + ((v[1] + v[5]) + (v[3] + v[7]));
  if constexpr (!L2) {
    // the reference build's dot tail: 4-wide products rounded on their own,
    // added in order, then a fused remainder
    for (; i + 4 <= n; i += 4)
      for (int l = 0; l < 4; ++l) {
        const float p = a[i + l] * b[i + l];
        s = s + p;
      }
  }
  for (; i < n; ++i) s = term<L2>(a[i], b[i], s);  // fused (contracted) tail
  return s;
}

template <bool L2>
float k_avx512(const float* a, const float* b, std::size_t n) noexcept {
  float acc[4][16] = {};
  std::size_t i = 0;
  for (; i + 64 <= n; i += 64)
    for (int j = 0; j < 4; ++j)
      for (int l = 0; l < 16; ++l) acc[j][l] = term<L2>(a[i + 16 * j + l], b[i + 16 * j + l], acc[j][l]);
  for (; i + 16 <= n; i += 16)
    for (int l = 0; l < 16; ++l) acc[0][l] = term<L2>(a[i + l], b[i + l], acc[0][l]);
  if (i < n) {
    float xa[16] = {}, xb[16] = {};
    for (std::size_t l = 0; l < n - i; ++l) {
      xa[l] = a[i + l];
      xb[l] = b[i + l];
    }
    for (int l = 0; l < 16; ++l) acc[1][l] = term<L2>(xa[l], xb[l], acc[1][l]);
  }
  float v[16];
  for (int l = 0; l < 16; ++l) v[l] = (acc[0][l] + acc[1][l]) + (acc[2][l] + acc[3][l]);
  float h8[8], h4[4];
  for (int l = 0; l < 8; ++l) h8[l] = v[8 + l] + v[l];
  for (int l = 0; l < 4; ++l) h4[l] = h8[4 + l] + h8[l];
  return (h4[0] + h4[2]) + (h4[1] + h4[3]);
}

template <bool L2>
float k_neon(const float* a, const float* b, std::size_t n) noexcept {
  float acc[4][4] = {};
  std::size_t i = 0;
  for (; i + 16 <= n; i += 16)
    for (int j = 0; j < 4; ++j)
      for (int l = 0; l < 4; ++l) acc[j][l] = term<L2>(a[i + 4 * j + l], b[i + 4 * j + l], acc[j][l]);
  for (; i + 4 <= n; i += 4)
    for (int l = 0; l < 4; ++l) acc[0][l] = term<L2>(a[i + l], b[i + l], acc[0][l]);
  float v[4];
  for (int l = 0; l < 4; ++l) v[l] = (acc[0][l] + acc[1][l]) + (acc[2][l] + acc[3][l]);
  float s = (v[0] + v[1]) + (v[2] + v[3]);
  for (; i < n; ++i) s = term<L2>(a[i], b[i], s);
  return s;
}

constexpr Kernels kTable[4] = {
    {Isa::Scalar, &k_scalar<true>, &k_scalar<false>},
    {Isa::AVX2, &k_avx2<true>, &k_avx2<false>},
    {Isa::AVX512, &k_avx512<true>, &k_avx512<false>},
    {Isa::NEON, &k_neon<true>, &k_neon<false>},
};

// The order the reference picks on this host: NEON on Arm (its only SIMD
// kernels there), AVX-512 on x86-64 (the widest; the GPU implements those
// two).  HNSW_SIMD names another, as it does for the reference.
const Kernels* initial() noexcept {
#if defined(__aarch64__)
  const Kernels* k = &kTable[3];
#else
  const Kernels* k = &kTable[2];
#endif
  if (const char* env = std::getenv("HNSW_SIMD"); env && *env) {  // NOLINT(concurrency-mt-unsafe)
    try {
      k = &kTable[static_cast<int>(parse_isa(env))];
    } catch (const std::exception&) {  // NOLINT(bugprone-empty-catch)
    }
  }
  return k;
}

std::atomic<const Kernels*>& active_ptr() noexcept {
  static std::atomic<const Kernels*> p{initial()};
  return p;
}

}  // namespace

float l2_sq_scalar(const float* a, const float* b, std::size_t dim) noexcept { return k_scalar<true>(a, b, dim); }
float dot_scalar(const float* a, const float* b, std::size_t dim) noexcept { return k_scalar<false>(a, b, dim); }

bool supported(Isa) noexcept { return true; }
const Kernels& active() noexcept { return *active_ptr().load(std::memory_order_acquire); }
const Kernels& get(Isa isa) { return kTable[static_cast<int>(isa)]; }
void set_active(Isa isa) { active_ptr().store(&kTable[static_cast<int>(isa)], std::memory_order_release); }

std::string_view isa_name(Isa isa) noexcept {
  switch (isa) {
    case Isa::Scalar: return "scalar";
    case Isa::AVX2: return "avx2";
    case Isa::AVX512: return "avx512";
    case Isa::NEON: return "neon";
  }
  return "unknown";
}

Isa parse_isa(std::string_view name) {
  if (name == "scalar") return Isa::Scalar;
  if (name == "avx2") return Isa::AVX2;
  if (name == "avx512") return Isa::AVX512;
  if (name == "neon") return Isa::NEON;
  throw std::invalid_argument("unknown ISA '" + std::string(name) + "'");
}

}  // namespace simd

// ---- filters (filter.hpp; reference src/filter.cpp:1-41) ----------------

FunctionFilter::FunctionFilter(std::function<bool(uint64_t)> fn) : fn_(std::move(fn)) {
  if (!fn_) throw std::invalid_argument("FunctionFilter: empty function");
}

BitsetFilter::BitsetFilter(uint64_t num_labels)
    : words_(static_cast<std::size_t>((num_labels + 63) / 64), 0), size_(num_labels) {}

BitsetFilter BitsetFilter::from_labels(const uint64_t* labels, std::size_t n) {
  uint64_t top = 0;
  for (std::size_t i = 0; i < n; ++i) top = labels[i] > top ? labels[i] : top;
  BitsetFilter f(n == 0 ? 0 : top + 1);
  for (std::size_t i = 0; i < n; ++i) f.set(labels[i]);
  return f;
}

void BitsetFilter::set(uint64_t label, bool value) {
  if (label >= size_) throw std::out_of_range("BitsetFilter::set: label out of range");
  const uint64_t bit = 1ULL << (label & 63);
  if (value) words_[label >> 6] |= bit;
  else words_[label >> 6] &= ~bit;
}

std::size_t BitsetFilter::count() const noexcept {
  std::size_t c = 0;
  for (uint64_t w : words_) c += static_cast<std::size_t>(__builtin_popcountll(w));
  return c;
}

}  // namespace hnsw
