#pragma once
// Metric names and the host distance-kernel registry of hnsw-gb300.
// Same declarations as the reference's include/hnsw/metric.hpp:1-61, so code
// written against hnsw-engine compiles unchanged.  The host kernels here are
// portable C++ reproducing each ISA's summation order (used by the CPU graph
// builder); queries run on the GPU, whose kernels reproduce the order selected
// with simd::set_active().

#include <cstddef>
#include <string>
#include <string_view>

namespace hnsw {

enum class Metric { L2, InnerProduct, Cosine };

/// Parse "l2" / "ip" / "inner_product" / "cosine" (case-sensitive). Throws std::invalid_argument.
Metric parse_metric(std::string_view name);
std::string_view metric_name(Metric m) noexcept;

namespace simd {

/// Summation orders of the reference's kernels.  All are available on every
/// host: they are reproduced in portable code, not executed with intrinsics.
enum class Isa { Scalar, AVX2, AVX512, NEON };

using DistanceFn = float (*)(const float* a, const float* b, std::size_t dim) noexcept;

struct Kernels {
  Isa isa;
  DistanceFn l2_sq;  ///< sum_i (a_i - b_i)^2
  DistanceFn dot;    ///< sum_i a_i * b_i
};

/// Order used by new/loaded indexes: AVX-512 unless HNSW_SIMD names another.
const Kernels& active() noexcept;
const Kernels& get(Isa isa);
bool supported(Isa isa) noexcept;
void set_active(Isa isa);
std::string_view isa_name(Isa isa) noexcept;
Isa parse_isa(std::string_view name);

float l2_sq_scalar(const float* a, const float* b, std::size_t dim) noexcept;
float dot_scalar(const float* a, const float* b, std::size_t dim) noexcept;

}  // namespace simd

inline float l2_sq(const float* a, const float* b, std::size_t dim) noexcept {
  return simd::active().l2_sq(a, b, dim);
}
inline float dot(const float* a, const float* b, std::size_t dim) noexcept { return simd::active().dot(a, b, dim); }

}  // namespace hnsw
