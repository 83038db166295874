// state.cpp -- hnsw::Index's host state: construction of an empty index,
// storage growth, and the accessors and mutations that are not searches or
// graph construction (include/hnsw/index.hpp:37-93).  Argument checks and
// exception types follow the reference's public contract
// (src/index.cpp:48-76, :247-330).
#include <algorithm>
#include <atomic>
#include <cmath>
#include <limits>
#include <stdexcept>
#include <string>
#include <unordered_set>

#include "graph.hpp"

namespace hnsw {

Index::Impl::Impl(const Params& p) : params(p) {
  if (p.dim == 0) throw std::invalid_argument("Index: dim must be > 0");
  if (p.M < 2) throw std::invalid_argument("Index: M must be >= 2");
  if (p.M > 2048) throw std::invalid_argument("Index: M must be <= 2048");
  if (p.ef_construction == 0) throw std::invalid_argument("Index: ef_construction must be > 0");
  if (p.max_elements > std::numeric_limits<uint32_t>::max() - 1)
    throw std::invalid_argument("Index: max_elements exceeds the 32-bit internal id space");
  dim = p.dim;
  padded_dim = gb::round_up(dim, gb::kPadFloats);
  M = p.M;
  M0 = 2 * p.M;
  // the construction beam is never narrower than a node's upper degree
  ef_construction = std::max(p.ef_construction, p.M);
  mL = 1.0 / std::log(static_cast<double>(M));
  l0_stride = 1 + M0;
  upper_stride = 1 + M;
  const simd::Kernels& k = simd::active();
  isa = k.isa;
  is_l2 = p.metric == Metric::L2;
  kernel = is_l2 ? k.l2_sq : k.dot;
  rng_state = p.seed;
  if (p.max_elements > 0) grow(p.max_elements);
}

Index::Impl::~Impl() {
  if (dev) hgd_graph_free(dev);
}

void Index::Impl::bind_pointers() {
  vecs = vec_store.data();
  l0 = l0_store.data();
  upper = upper_store.data();
  labels = label_store.data();
  levels = level_store.data();
}

void Index::Impl::grow(std::size_t n) {
  if (n <= capacity) return;
  if (read_only) throw std::runtime_error("index is read-only (memory-mapped)");
  if (n > std::numeric_limits<uint32_t>::max() - 1)
    throw std::runtime_error("Index: capacity exceeds the 32-bit internal id space");
  vec_store.resize(n * padded_dim, 0.0f);
  l0_store.resize(n * l0_stride, 0u);
  label_store.resize(n, 0);
  level_store.resize(n, 0);
  upper_offset.resize(n, 0);
  deleted.resize(n, 0);
  capacity = n;
  bind_pointers();
}

Index::Index(const Params& params) : impl_(std::make_unique<Impl>(params)) {}
Index::Index(std::unique_ptr<Impl> impl) : impl_(std::move(impl)) {}
Index::~Index() = default;
Index::Index(Index&&) noexcept = default;
Index& Index::operator=(Index&&) noexcept = default;

void Index::add(const float* vec, uint64_t label) { add_batch(vec, &label, 1, 1); }

namespace {
// every label is checked before the index changes: new, and once per batch
void check_new_labels(const Index::Impl& im, const uint64_t* labels, std::size_t n) {
  if (im.read_only) throw std::runtime_error("index is read-only (memory-mapped); load without mmap to modify");
  std::unordered_set<uint64_t> batch;
  batch.reserve(n);
  for (std::size_t i = 0; i < n; ++i) {
    if (im.label_to_id.count(labels[i]) != 0)
      throw std::invalid_argument("add: label " + std::to_string(labels[i]) + " already exists");
    if (!batch.insert(labels[i]).second)
      throw std::invalid_argument("add_batch: duplicate label " + std::to_string(labels[i]) + " in batch");
  }
}
}  // namespace

void Index::add_batch(const float* vecs, const uint64_t* labels, std::size_t n, std::size_t num_threads) {
  if (n == 0) return;
  if (vecs == nullptr || labels == nullptr) throw std::invalid_argument("add_batch: null input");
  std::unique_lock<std::shared_mutex> lk(impl_->api_mutex);
  Impl& im = *impl_;
  check_new_labels(im, labels, n);
  gb::insert_batch(im, vecs, labels, n, num_threads);
  std::lock_guard<std::mutex> g(im.dev_mutex);
  im.dev_stale = true;
}

GpuBuildStats Index::add_batch_gpu(const float* vecs, const uint64_t* labels, std::size_t n,
                                   const GpuBuildOptions& opt) {
  if (n == 0) return {};
  if (vecs == nullptr || labels == nullptr) throw std::invalid_argument("add_batch: null input");
  std::unique_lock<std::shared_mutex> lk(impl_->api_mutex);
  Impl& im = *impl_;
  check_new_labels(im, labels, n);
  const GpuBuildStats st = gb::insert_batch_gpu(im, vecs, labels, n, opt);
  std::lock_guard<std::mutex> g(im.dev_mutex);
  im.dev_stale = true;
  return st;
}

void Index::mark_deleted(uint64_t label) {
  std::unique_lock<std::shared_mutex> lk(impl_->api_mutex);
  Impl& im = *impl_;
  const auto it = im.label_to_id.find(label);
  if (it == im.label_to_id.end()) throw std::invalid_argument("mark_deleted: unknown label " + std::to_string(label));
  const uint32_t id = it->second;
  if (im.deleted[id] != 0) return;
  im.deleted[id] = 1;
  ++im.num_deleted;
  // a resident mirror gets the one tombstone bit; a stale one is rebuilt anyway
  std::lock_guard<std::mutex> g(im.dev_mutex);
  if (im.dev && !im.dev_stale && hgd_graph_set_deleted(im.dev, id, 1) != HGD_OK)
    throw std::runtime_error(std::string("mark_deleted: ") + hgd_last_error());
}

bool Index::is_deleted(uint64_t label) const {
  std::shared_lock<std::shared_mutex> lk(impl_->api_mutex);
  const auto it = impl_->label_to_id.find(label);
  return it != impl_->label_to_id.end() && impl_->deleted[it->second] != 0;
}

bool Index::contains(uint64_t label) const {
  std::shared_lock<std::shared_mutex> lk(impl_->api_mutex);
  return impl_->label_to_id.find(label) != impl_->label_to_id.end();
}

std::size_t Index::size() const {
  std::shared_lock<std::shared_mutex> lk(impl_->api_mutex);
  return impl_->count;
}
std::size_t Index::dim() const noexcept { return impl_->dim; }
Metric Index::metric() const noexcept { return impl_->params.metric; }
const Params& Index::params() const noexcept { return impl_->params; }
std::size_t Index::capacity() const {
  std::shared_lock<std::shared_mutex> lk(impl_->api_mutex);
  return impl_->capacity;
}
std::size_t Index::ef() const {
  std::shared_lock<std::shared_mutex> lk(impl_->api_mutex);
  return impl_->ef_search;
}
void Index::set_ef(std::size_t ef) {
  if (ef == 0) throw std::invalid_argument("set_ef: ef must be > 0");
  std::unique_lock<std::shared_mutex> lk(impl_->api_mutex);
  impl_->ef_search = ef;
}
int Index::max_level() const {
  std::shared_lock<std::shared_mutex> lk(impl_->api_mutex);
  return impl_->max_level;
}
bool Index::read_only() const noexcept { return impl_->read_only; }

std::size_t Index::memory_usage() const {
  std::shared_lock<std::shared_mutex> lk(impl_->api_mutex);
  const Impl& im = *impl_;
  const std::size_t per_node = im.padded_dim * sizeof(float) + im.l0_stride * sizeof(uint32_t) +
                               2 * sizeof(uint64_t) + sizeof(uint8_t) * 2;
  return im.count * per_node + im.upper_used * sizeof(uint32_t);
}

std::vector<float> Index::get_vector(uint64_t label) const {
  std::shared_lock<std::shared_mutex> lk(impl_->api_mutex);
  const auto it = impl_->label_to_id.find(label);
  if (it == impl_->label_to_id.end()) throw std::invalid_argument("get_vector: unknown label");
  const float* v = impl_->vec(it->second);
  return std::vector<float>(v, v + impl_->dim);
}

namespace tuning {
namespace {
std::atomic<bool> g_prefetch{true};
}
// kept for API compatibility: the GPU walk has no software-prefetch switch
void set_prefetch(bool enabled) noexcept { g_prefetch.store(enabled); }
bool prefetch_enabled() noexcept { return g_prefetch.load(); }
}  // namespace tuning

}  // namespace hnsw
