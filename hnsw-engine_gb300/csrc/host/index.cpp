// index.cpp -- hnsw::Index queries: the graph is mirrored into HBM once and
// every search / search_batch is answered by the CUDA kernels behind the
// hgd_* C ABI.  There is no CPU search path: if the mirror cannot be built
// or a launch fails, the call throws.
//
// Semantics kept from the reference (src/search_layer.cpp:173-194):
//   k == 0 -> invalid_argument; nq == 0 -> no-op; null pointers ->
//   invalid_argument; ef == 0 -> the index's set_ef value; ef < k -> k;
//   search() returns min(k, #eligible) results, search_batch() pads rows
//   with {kInvalidLabel, +inf}.
#include <cstring>
#include <limits>
#include <shared_mutex>
#include <stdexcept>
#include <string>

#include "graph.hpp"

namespace hnsw {

static_assert(sizeof(Neighbor) == 16, "device records are 16 bytes");

using gb::FilterBits;
using gb::to_bits;

namespace {

int order_of(simd::Isa isa) {
  switch (isa) {
    case simd::Isa::Scalar: return HGD_ORDER_SCALAR;
    case simd::Isa::AVX2: return HGD_ORDER_AVX2;
    case simd::Isa::AVX512: return HGD_ORDER_AVX512;
    case simd::Isa::NEON: return HGD_ORDER_NEON;
  }
  return HGD_ORDER_AVX512;
}

[[noreturn]] void rethrow(int rc, const char* what) {
  const std::string msg = std::string(what) + ": " + hgd_last_error();
  if (rc == HGD_EINVAL) throw std::invalid_argument(msg);
  throw std::runtime_error(msg);
}

}  // namespace

hgd_graph_view Index::Impl::device_view() const {
  hgd_graph_view v{};
  v.count = count;
  v.dim = dim;
  v.padded_dim = padded_dim;
  v.M = M;
  v.metric = static_cast<int32_t>(params.metric);
  v.max_level = max_level;
  v.entry_point = entry_point;
  v.vectors = vecs;
  v.level0 = l0;
  v.upper = upper;
  v.upper_used = upper_used;
  v.upper_offset = upper_offset.data();
  v.labels = labels;
  v.levels = levels;
  v.deleted = deleted.data();
  return v;
}

int Index::Impl::device_order() const { return order_of(isa); }

hgd_graph* Index::Impl::device_graph() const {
  std::lock_guard<std::mutex> g(dev_mutex);
  if (dev && !dev_stale) return dev;
  if (dev) {
    hgd_graph_free(dev);
    dev = nullptr;
  }
  const hgd_graph_view v = device_view();
  hgd_graph* out = nullptr;
  const int rc = hgd_graph_upload(&v, device, order_of(isa), &out);
  if (rc != HGD_OK) rethrow(rc, "upload to GPU");
  if (!tuning.empty()) hgd_graph_set_tuning(out, tuning.data(), static_cast<uint32_t>(tuning.size()));
  hgd_graph_set_launch_mode(out, launch_mode);
  dev = out;
  dev_stale = false;
  return dev;
}

void Index::set_device(int device) {
  std::unique_lock<std::shared_mutex> lk(impl_->api_mutex);
  std::lock_guard<std::mutex> g(impl_->dev_mutex);
  if (impl_->device != device) {
    impl_->device = device;
    impl_->dev_stale = true;
  }
}

void Index::search_batch_ex(const float* qs, std::size_t nq, std::size_t k, std::size_t ef, Neighbor* out,
                            const SearchOptions& opt) const {
  if (k == 0) throw std::invalid_argument("search_batch: k must be > 0");
  if (nq == 0) return;
  if (qs == nullptr || out == nullptr) throw std::invalid_argument("search_batch: null pointer");
  if (k > std::numeric_limits<uint32_t>::max() || ef > std::numeric_limits<uint32_t>::max())
    throw std::invalid_argument("search_batch: k / ef out of range");
  std::shared_lock<std::shared_mutex> lk(impl_->api_mutex);
  const Impl& im = *impl_;
  if (im.count == 0) {
    if (opt.out_on_device) throw std::invalid_argument("search_batch: empty index with a device output buffer");
    for (std::size_t i = 0; i < nq * k; ++i) out[i] = Neighbor{kInvalidLabel, std::numeric_limits<float>::infinity()};
    return;
  }
  hgd_graph* g = im.device_graph();
  std::vector<FilterBits> fb(opt.num_filters);
  std::vector<hgd_bitset> views(opt.num_filters);
  for (std::size_t i = 0; i < opt.num_filters; ++i) {
    if (opt.filters[i] == nullptr) throw std::invalid_argument("search_batch: null filter in table");
    to_bits(im, opt.filters[i], fb[i]);
    views[i] = fb[i].view;
  }
  hgd_search_args a{};
  a.queries = qs;
  a.nq = nq;
  a.k = static_cast<uint32_t>(k);
  a.ef = static_cast<uint32_t>(ef);
  a.ef_default = static_cast<uint32_t>(std::min<std::size_t>(im.ef_search, std::numeric_limits<uint32_t>::max()));
  a.precision = static_cast<uint32_t>(opt.precision);
  a.ef_per_query = opt.ef_per_query;
  a.k_per_query = opt.k_per_query;
  a.filters = views.empty() ? nullptr : views.data();
  a.num_filters = static_cast<uint32_t>(views.size());
  a.filter_of_query = opt.filter_of_query;
  a.out = out;
  a.stream = opt.stream;
  a.counters = opt.counters;
  a.queries_on_device = opt.queries_on_device ? 1 : 0;
  a.out_on_device = opt.out_on_device ? 1 : 0;
  a.synchronize = opt.out_on_device ? 0 : 1;
  a.use_graph = opt.use_graph ? 1 : 0;
  a.filter_scan_permille = opt.filter_scan_permille;
  a.rerank_factor = opt.rerank_factor;
  a.warps_per_query = opt.warps_per_query;
  a.lists_per_step = opt.lists_per_step;
  a.filter_scan_mode = opt.filter_scan_mode;
  a.hash_slots = opt.hash_slots;
  a.cand_cap = opt.cand_cap;
  a.warps_per_block = opt.warps_per_block;
  a.pool_cap = opt.pool_cap;
  const int rc = hgd_search(g, &a);
  if (rc != HGD_OK) rethrow(rc, "search_batch");
}

void Index::search_batch(const float* qs, std::size_t nq, std::size_t k, std::size_t ef, Neighbor* out,
                         std::size_t /*num_threads*/, const Filter* f) const {
  SearchOptions opt;
  const Filter* table[1] = {f};
  if (f != nullptr) {
    opt.filters = table;
    opt.num_filters = 1;
  }
  search_batch_ex(qs, nq, k, ef, out, opt);
}

std::vector<Neighbor> Index::search(const float* q, std::size_t k, std::size_t ef, const Filter* f) const {
  if (k == 0) throw std::invalid_argument("search: k must be > 0");
  if (q == nullptr) throw std::invalid_argument("search: null query");
  std::vector<Neighbor> out(k);
  std::vector<uint32_t> nres(1, 0);
  // one query through the batch path; the row's result count comes back in nres
  std::shared_lock<std::shared_mutex> lk(impl_->api_mutex);
  const Impl& im = *impl_;
  if (im.count == 0) return {};
  hgd_graph* g = im.device_graph();
  FilterBits fb;
  hgd_bitset view{};
  if (f) {
    to_bits(im, f, fb);
    view = fb.view;
  }
  hgd_search_args a{};
  a.queries = q;
  a.nq = 1;
  a.k = static_cast<uint32_t>(k);
  a.ef = static_cast<uint32_t>(std::min<std::size_t>(ef, std::numeric_limits<uint32_t>::max()));
  a.ef_default = static_cast<uint32_t>(std::min<std::size_t>(im.ef_search, std::numeric_limits<uint32_t>::max()));
  a.filters = f ? &view : nullptr;
  a.num_filters = f ? 1 : 0;
  a.out = out.data();
  a.nres = nres.data();
  a.synchronize = 1;
  const int rc = hgd_search(g, &a);
  if (rc != HGD_OK) rethrow(rc, "search");
  out.resize(nres[0]);
  return out;
}

}  // namespace hnsw
