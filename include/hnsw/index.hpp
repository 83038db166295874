#pragma once
// hnsw::Index for GB300: the reference's public C++ API
// (include/hnsw/index.hpp:14-118) with queries answered on the GPU.
//
// The graph lives in host memory exactly as the reference lays it out
// (FORMAT v1 sections) and is mirrored into HBM on first use; mutations
// (add, mark_deleted) update the mirror before the next search.  search /
// search_batch run the greedy descent and layer-0 beam search as CUDA
// kernels and return the reference's ids and distances.

#include <cstddef>
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "hnsw/filter.hpp"
#include "hnsw/metric.hpp"

namespace hnsw {

struct Params {
  std::size_t dim = 0;
  Metric metric = Metric::L2;
  std::size_t M = 16;
  std::size_t ef_construction = 200;
  std::size_t max_elements = 0;  ///< 0 = grow geometrically
  uint64_t seed = 100;
};

struct Neighbor {
  uint64_t label;
  float distance;
};

inline constexpr uint64_t kInvalidLabel = ~uint64_t{0};

/// Options beyond the reference's signature, for batched/served callers.
struct SearchOptions {
  const uint32_t* ef_per_query = nullptr;  ///< nq entries (host), overrides ef
  const uint32_t* k_per_query = nullptr;   ///< nq entries (host), each <= k
  const Filter* const* filters = nullptr;  ///< per-query filter table
  std::size_t num_filters = 0;
  const int32_t* filter_of_query = nullptr;  ///< nq entries, -1 = none
  void* stream = nullptr;                    ///< cudaStream_t; nullptr = the index's own stream
  int precision = 0;                         ///< 0 fp32, 1 fp16, 2 fp8 (traversal; exact fp32 rerank)
  uint64_t* counters = nullptr;              ///< optional nq x 8 traversal counters
  // launch shape (0 = automatic): visited-hash slots, candidate head
  // capacity, warps per block, spill-pool entries per warp
  uint32_t hash_slots = 0, cand_cap = 0, warps_per_block = 0, pool_cap = 0;
  /// device-resident batches: queries / ef / k (and out) are device pointers;
  /// with out_on_device the call only enqueues work on `stream`.
  bool queries_on_device = false, out_on_device = false;
  /// device-resident batches without filters or counters: capture the launch
  /// sequence into a CUDA graph (second call of a shape) and replay it
  bool use_graph = false;
  /// FP16 / FP8 batches: queries whose filter allows at most this many per
  /// mille of the nodes are answered by the exact tensor-core scan (0: off)
  uint32_t filter_scan_permille = 0;
  /// FP16 / FP8 batches: the exact FP32 rerank covers the best
  /// rerank_factor x k entries of the traversal pool (at least 32); 0 = all
  uint32_t rerank_factor = 0;
  /// FP16 / FP8 batches with dim <= 128: 4 = four warps walk each query (a
  /// beam search: lower latency, not the reference's visit order); 1 = one
  uint32_t warps_per_query = 1;
  /// FP16 / FP8 batches with dim <= 128: 1..4 = one warp walks each query as
  /// a beam search expanding this many neighbour lists per step, with row
  /// distances on the tensor cores (throughput; not the reference's visit
  /// order); 0 = the one-warp walk in the reference's order
  uint32_t lists_per_step = 0;
  /// the exact scan of routed queries: 0 auto (fewer bytes), 1 only the
  /// rows the filter allows, 2 every row (the tcgen05 GEMM)
  uint32_t filter_scan_mode = 0;
};

/// Graph construction on the GPU (Index::add_batch_gpu; no counterpart in
/// the reference).  New nodes are linked in waves that search the graph
/// built so far, one warp per node; a wave holds at most wave_fraction of the
/// nodes already linked (at least wave_min, at most wave_max).
struct GpuBuildOptions {
  int device = -1;             ///< CUDA device; -1 = the index's (set_device)
  double wave_fraction = 0.0;  ///< 0 = 0.02
  uint32_t wave_min = 0;       ///< 0 = 1
  uint32_t wave_max = 0;       ///< 0 = four (peers: sixteen) times the warps the GPU keeps resident
  /// each new node re-chooses its list among the nodes of its wave that
  /// chose the same neighbours (links a wave's nodes to each other)
  bool peers = false;
};
struct GpuBuildStats {
  uint32_t waves = 0;                ///< kernel waves launched
  uint64_t dropped_proposals = 0;    ///< reverse edges beyond a list's per-wave inbox
  double seconds = 0.0;              ///< wall time of the GPU linking (upload to download)
};

class Index {
 public:
  explicit Index(const Params& params);
  ~Index();
  Index(Index&&) noexcept;
  Index& operator=(Index&&) noexcept;
  Index(const Index&) = delete;
  Index& operator=(const Index&) = delete;

  void add(const float* vec, uint64_t label);
  void add_batch(const float* vecs, const uint64_t* labels, std::size_t n, std::size_t num_threads = 0);
  /// add_batch with the linking on the GPU (no counterpart in the reference;
  /// replaces src/index.cpp:273-306's parallel link loop).  The same
  /// validation, errors, stored rows, labels and levels as add_batch; the
  /// graph differs from a CPU build's (as a threaded build's does) and is
  /// judged on recall.  Limits: size() + n < 2^24, M <= 32, dim <= 1024,
  /// ef_construction <= 1024 (std::invalid_argument beyond them).
  GpuBuildStats add_batch_gpu(const float* vecs, const uint64_t* labels, std::size_t n,
                              const GpuBuildOptions& opt = {});

  std::vector<Neighbor> search(const float* q, std::size_t k, std::size_t ef = 0, const Filter* f = nullptr) const;
  /// num_threads is accepted for source compatibility; the GPU runs all queries.
  void search_batch(const float* qs, std::size_t nq, std::size_t k, std::size_t ef, Neighbor* out,
                    std::size_t num_threads = 0, const Filter* f = nullptr) const;
  /// Batched search with per-query ef / k / filter and an explicit stream.
  void search_batch_ex(const float* qs, std::size_t nq, std::size_t k, std::size_t ef, Neighbor* out,
                       const SearchOptions& opt) const;

  void mark_deleted(uint64_t label);
  bool is_deleted(uint64_t label) const;
  bool contains(uint64_t label) const;

  std::size_t size() const;
  std::size_t dim() const noexcept;
  Metric metric() const noexcept;
  const Params& params() const noexcept;
  std::size_t capacity() const;
  std::size_t ef() const;
  void set_ef(std::size_t ef);
  int max_level() const;
  bool read_only() const noexcept;
  std::size_t memory_usage() const;
  std::vector<float> get_vector(uint64_t label) const;

  void save(const std::string& path) const;
  static Index load(const std::string& path, bool mmap = false);
  /// load() with the device graph built in the same pass (no counterpart in
  /// the reference): the vectors, layer 0 and labels are streamed to `device`
  /// through pinned staging buffers while the file is read and hashed, and
  /// layer 0 is laid out on the device.  Same validation and errors as
  /// load(); mmap = true keeps the host arrays in the read-only mapping.
  static Index load_to_device(const std::string& path, int device, bool mmap = false);

  /// CUDA device the graph is mirrored to (default 0); call before the first search.
  void set_device(int device);

  struct Impl;
  Impl* impl() const noexcept { return impl_.get(); }

 private:
  explicit Index(std::unique_ptr<Impl> impl);
  std::unique_ptr<Impl> impl_;
};

namespace tuning {
/// Kept for source compatibility with the reference's ablation switch (the
/// GPU kernels overlap gathers through warps, not software prefetch).
void set_prefetch(bool enabled) noexcept;
bool prefetch_enabled() noexcept;
}  // namespace tuning

/// Exact search over all vectors (ground truth), on the GPU.
class BruteForceIndex {
 public:
  BruteForceIndex(std::size_t dim, Metric metric);
  ~BruteForceIndex();
  BruteForceIndex(BruteForceIndex&&) noexcept;
  BruteForceIndex& operator=(BruteForceIndex&&) noexcept;
  void add(const float* vecs, const uint64_t* labels, std::size_t n);
  std::vector<Neighbor> search(const float* q, std::size_t k, const Filter* f = nullptr) const;
  void search_batch(const float* qs, std::size_t nq, std::size_t k, Neighbor* out, std::size_t num_threads = 0,
                    const Filter* f = nullptr) const;
  std::size_t size() const noexcept { return labels_.size(); }
  std::size_t dim() const noexcept { return dim_; }
  // GPU kernel choice (0 auto, 1 CUDA-core scan, 2 tensor-core GEMM + exact
  // rerank) and the one that answered the last search; no counterpart in the
  // reference.
  void set_gpu_path(int path);
  int last_gpu_path() const noexcept { return last_path_; }

  struct Dev;

 private:
  std::size_t dim_;
  Metric metric_;
  std::vector<float> data_;
  std::vector<uint64_t> labels_;
  mutable std::unique_ptr<Dev> dev_;
  int path_ = 0;
  mutable int last_path_ = 0;
};

}  // namespace hnsw
