// graph.hpp -- host state behind hnsw::Index.
//
// The arrays are those of the reference's Index::Impl
// (src/index_impl.hpp:193-214) and of FORMAT v1, so a loaded file can be
// re-saved byte for byte and uploaded to HBM without conversion:
//   vectors   count x padded_dim float32 (64-byte aligned rows, zero tail)
//   level0    count x (1 + 2M) uint32  [n, ids...]
//   upper     per node with level L >= 1: L blocks of (1 + M) uint32
//   labels    count x uint64;  levels count x uint8;  deleted count x uint8
#pragma once

#include <atomic>
#include <cstddef>
#include <cstdint>
#include <memory>
#include <mutex>
#include <new>
#include <shared_mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "hnsw/index.hpp"
#include "hnswgpu.h"
#include "hnswgpu_device.h"

namespace hnsw::gb {

inline constexpr std::size_t kRowAlign = 64;  // bytes; rows are padded to 16 floats
inline constexpr std::size_t kPadFloats = 16;
inline constexpr uint32_t kNoNode = ~uint32_t{0};
inline constexpr int kMaxLevel = 64;
inline constexpr std::size_t kStripes = 4096;

inline std::size_t round_up(std::size_t v, std::size_t m) { return (v + m - 1) / m * m; }

template <typename T>
struct Aligned64 {
  using value_type = T;
  Aligned64() noexcept = default;
  template <typename U>
  Aligned64(const Aligned64<U>&) noexcept {}  // NOLINT
  T* allocate(std::size_t n) {
    if (n == 0) return nullptr;
    return static_cast<T*>(::operator new(round_up(n * sizeof(T), kRowAlign), std::align_val_t{kRowAlign}));
  }
  void deallocate(T* p, std::size_t) noexcept { ::operator delete(p, std::align_val_t{kRowAlign}); }
  template <typename U>
  bool operator==(const Aligned64<U>&) const noexcept {
    return true;
  }
};

/// (distance, internal id) with the reference's total order (index_impl.hpp:58-71).
struct Cand {
  float dist;
  uint32_t id;
};
inline bool closer(const Cand& a, const Cand& b) noexcept {
  return a.dist < b.dist || (a.dist == b.dist && a.id < b.id);
}
struct CloserFirst {  // heap comparator: max-heap on (dist, id)
  bool operator()(const Cand& a, const Cand& b) const noexcept { return closer(a, b); }
};
struct FartherFirst {  // heap comparator: min-heap on (dist, id)
  bool operator()(const Cand& a, const Cand& b) const noexcept { return closer(b, a); }
};

/// Read-only file mapping (load with mmap = true).
class Mapping {
 public:
  Mapping() = default;
  explicit Mapping(const std::string& path);
  ~Mapping();
  Mapping(Mapping&& o) noexcept;
  Mapping& operator=(Mapping&& o) noexcept;
  Mapping(const Mapping&) = delete;
  Mapping& operator=(const Mapping&) = delete;
  const unsigned char* data() const noexcept { return data_; }
  std::size_t size() const noexcept { return size_; }

 private:
  void reset() noexcept;
  const unsigned char* data_ = nullptr;
  std::size_t size_ = 0;
};

}  // namespace hnsw::gb

namespace hnsw {

struct Index::Impl {
  Params params;
  std::size_t dim = 0, padded_dim = 0, M = 0, M0 = 0, ef_construction = 0, ef_search = 10;
  double mL = 0.0;
  std::size_t l0_stride = 0, upper_stride = 0;
  simd::Isa isa = simd::Isa::AVX512;
  simd::DistanceFn kernel = nullptr;
  bool is_l2 = true;

  std::vector<float, gb::Aligned64<float>> vec_store;
  std::vector<uint32_t, gb::Aligned64<uint32_t>> l0_store;
  std::vector<uint32_t> upper_store;
  std::vector<uint64_t> label_store;
  std::vector<uint8_t> level_store;
  const float* vecs = nullptr;
  uint32_t* l0 = nullptr;
  uint32_t* upper = nullptr;
  const uint64_t* labels = nullptr;
  const uint8_t* levels = nullptr;

  std::vector<uint64_t> upper_offset;
  std::vector<uint8_t> deleted;
  std::size_t num_deleted = 0;
  std::unordered_map<uint64_t, uint32_t> label_to_id;
  std::size_t count = 0, capacity = 0, upper_used = 0;
  uint32_t entry_point = gb::kNoNode;
  int max_level = -1;
  uint64_t rng_state = 0;
  gb::Mapping mapping;
  bool read_only = false;

  mutable std::shared_mutex api_mutex;
  std::mutex top_mutex;  // entry point and top level during construction
  std::unique_ptr<std::mutex[]> stripes{new std::mutex[gb::kStripes]};

  // GPU mirror (rebuilt lazily after add; tombstones are patched in place)
  int device = 0;
  mutable std::mutex dev_mutex;
  mutable hgd_graph* dev = nullptr;
  mutable bool dev_stale = true;
  std::vector<hgd_tune_entry> tuning;  // launch shapes per ef bucket (autotuner), re-applied on upload
  int launch_mode = HGD_LAUNCH_BUCKETS;  // per-bucket launches or one largest-ef-first launch

  explicit Impl(const Params& p);
  ~Impl();

  float dist(const float* a, const float* b) const noexcept {
    const float r = kernel(a, b, padded_dim);
    return is_l2 ? r : 1.0f - r;
  }
  const float* vec(uint32_t id) const noexcept { return vecs + std::size_t{id} * padded_dim; }
  uint32_t* list0(uint32_t id) const noexcept { return l0 + std::size_t{id} * l0_stride; }
  uint32_t* list(uint32_t id, int level) const noexcept {
    return level == 0 ? list0(id) : upper + upper_offset[id] + std::size_t(level - 1) * upper_stride;
  }
  std::size_t degree_cap(int level) const noexcept { return level == 0 ? M0 : M; }
  std::mutex& lock_of(uint32_t id) const noexcept { return stripes[id & (gb::kStripes - 1)]; }
  void bind_pointers();
  void grow(std::size_t n);

  // device mirror (index.cpp)
  hgd_graph* device_graph() const;
  hgd_graph_view device_view() const;  // the host arrays, as the device upload reads them
  int device_order() const;            // HGD_ORDER_* of the distance kernel in use
};

}  // namespace hnsw

namespace hnsw::gb {

/// Filter -> device bitset.  BitsetFilter ships its label-space words; any
/// other filter is evaluated once per node on the host (it is a predicate on
/// labels, so this is the same decision the reference makes lazily).
struct FilterBits {
  std::vector<uint64_t> owned;
  hgd_bitset view{};
};

inline void to_bits(const Index::Impl& im, const Filter* f, FilterBits& out) {
  if (const auto* bs = dynamic_cast<const BitsetFilter*>(f)) {
    out.view.words = bs->words();
    out.view.num_bits = bs->size();
    out.view.label_space = 1;
    return;
  }
  out.owned.assign((im.count + 63) / 64, 0);
  for (std::size_t i = 0; i < im.count; ++i)
    if (f->allowed(im.labels[i])) out.owned[i >> 6] |= 1ULL << (i & 63);
  out.view.words = out.owned.data();
  out.view.num_bits = im.count;
  out.view.label_space = 0;
}


}  // namespace hnsw::gb

namespace hnsw::gb {

// CPU graph construction (build.cpp): stores a validated batch and links it
// into the graph with `threads` workers (0 = all hardware threads)
void insert_batch(Index::Impl& g, const float* vecs, const uint64_t* labels, std::size_t n, std::size_t threads);
// GPU graph construction (build.cpp + build_graph.cu): stores the batch as
// insert_batch does, then links it on the GPU; on failure the index is left
// as it was
GpuBuildStats insert_batch_gpu(Index::Impl& g, const float* vecs, const uint64_t* labels, std::size_t n,
                               const GpuBuildOptions& opt);

// launch-shape autotuner (tune.cpp): times candidate shapes per ef bucket on
// a sample of queries, installs the fastest and returns the table as JSON
std::string autotune(Index::Impl& im, const float* queries, size_t nq, uint32_t k, uint32_t ef_max, int precision,
                     const uint32_t* ef_per_query);
// installs a table written by autotune (entries of other graphs' devices are
// kept: the shape fields are valid on any GPU)
void apply_tuning_json(Index::Impl& im, const std::string& json);

// continuous-batching server (server.cpp)
class Server;
Server* server_new(const Index::Impl& im, const hg_server_config& cfg);
void server_delete(Server* s);
uint64_t server_submit(Server* s, const hg_request& r);
void server_wait(Server* s, uint64_t ticket, double* latency_ms);
void server_replay(Server* s, const hg_request* reqs, const double* arrival_s, size_t n, hg_server_stats* out,
                   double* latency_ms);
void server_stats(Server* s, hg_server_stats* out);

}  // namespace hnsw::gb
