// build.cpp -- graph construction on the host CPU (Malkov & Yashunin Alg. 1
// with the Alg. 4 heuristic), restating the reference's add/add_batch
// (src/index.cpp:48-306) and its locked layer search
// (src/search_layer.cpp:29-134, Locked = true).
//
// Construction is not on the GPU path: it produces the graph that the query
// kernels traverse, exactly as the reference's add_batch would.  With one
// thread the result is deterministic and byte-identical to the reference's
// single-threaded build on a host using the same distance order; with more
// threads it is as nondeterministic as the reference's parallel build.
#include <algorithm>
#include <cmath>
#include <exception>
#include <limits>
#include <stdexcept>
#include <string>
#include <thread>
#include <unordered_set>

#include "graph.hpp"

namespace hnsw {

using gb::Cand;
using gb::CloserFirst;
using gb::FartherFirst;

namespace {

/// splitmix64: portable level generator (index.cpp:20-28).
inline uint64_t splitmix64(uint64_t& s) noexcept {
  uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

/// prepare_vector (space.hpp:31-40): copy, or scale to unit length for cosine.
void prepare(Metric m, const float* src, float* dst, std::size_t dim) {
  if (m != Metric::Cosine) {
    std::copy(src, src + dim, dst);
    return;
  }
  double norm = 0.0;
  for (std::size_t i = 0; i < dim; ++i) norm += static_cast<double>(src[i]) * src[i];
  const float inv = norm > 0.0 ? static_cast<float>(1.0 / std::sqrt(norm)) : 1.0f;
  for (std::size_t i = 0; i < dim; ++i) dst[i] = src[i] * inv;
}

/// Work sharing over [0, n) with the first exception rethrown after join
/// (threadpool.cpp:18-52).
template <typename Fn>
void parallel_range(std::size_t n, std::size_t threads, Fn&& fn) {
  if (n == 0) return;
  if (threads == 0) {
    const unsigned hw = std::thread::hardware_concurrency();
    threads = hw ? hw : 1;
  }
  threads = std::min(threads, n);
  if (threads == 1) {
    for (std::size_t i = 0; i < n; ++i) fn(i);
    return;
  }
  std::atomic<std::size_t> next{0};
  std::atomic<bool> failed{false};
  std::exception_ptr err;
  std::mutex err_mu;
  auto worker = [&]() {
    try {
      while (!failed.load(std::memory_order_relaxed)) {
        const std::size_t i = next.fetch_add(1, std::memory_order_relaxed);
        if (i >= n) break;
        fn(i);
      }
    } catch (...) {
      std::lock_guard<std::mutex> g(err_mu);
      if (!err) err = std::current_exception();
      failed.store(true);
    }
  };
  std::vector<std::thread> pool;
  pool.reserve(threads - 1);
  for (std::size_t t = 1; t < threads; ++t) pool.emplace_back(worker);
  worker();
  for (auto& t : pool) t.join();
  if (err) std::rethrow_exception(err);
}

/// Copy of a neighbour list taken under its stripe lock.
void snapshot(const Index::Impl& im, uint32_t id, int level, std::vector<uint32_t>& out) {
  std::lock_guard<std::mutex> g(im.lock_of(id));
  const uint32_t* l = im.list(id, level);
  out.assign(l + 1, l + 1 + l[0]);
}

/// Greedy single-best descent on one layer (first strict improvement wins).
Cand descend(const Index::Impl& im, const float* q, Cand cur, int level, std::vector<uint32_t>& buf) {
  for (bool moved = true; moved;) {
    moved = false;
    snapshot(im, cur.id, level, buf);
    for (uint32_t nb : buf) {
      const float d = im.dist(q, im.vec(nb));
      if (d < cur.dist) {
        cur = Cand{d, nb};
        moved = true;
      }
    }
  }
  return cur;
}

/// Beam search on one layer from several entry points (Alg. 2, unfiltered);
/// leaves the ef best in s.res as a heap.
void beam(const Index::Impl& im, const float* q, const std::vector<Cand>& eps, std::size_t ef, int level,
          gb::BuildScratch& s) {
  s.begin(im.capacity);
  auto& cand = s.cand;
  auto& res = s.res;
  cand.clear();
  res.clear();
  for (const Cand& e : eps) {
    if (s.mark[e.id] == s.epoch) continue;
    s.mark[e.id] = s.epoch;
    cand.push_back(e);
    res.push_back(e);
  }
  std::make_heap(cand.begin(), cand.end(), FartherFirst{});
  std::make_heap(res.begin(), res.end(), CloserFirst{});
  while (res.size() > ef) {
    std::pop_heap(res.begin(), res.end(), CloserFirst{});
    res.pop_back();
  }
  while (!cand.empty()) {
    const Cand c = cand.front();
    if (res.size() >= ef && c.dist > res.front().dist) break;
    std::pop_heap(cand.begin(), cand.end(), FartherFirst{});
    cand.pop_back();
    snapshot(im, c.id, level, s.nbuf);
    for (uint32_t id : s.nbuf) {
      if (s.mark[id] == s.epoch) continue;
      s.mark[id] = s.epoch;
      const float d = im.dist(q, im.vec(id));
      if (res.size() < ef || d < res.front().dist) {
        cand.push_back(Cand{d, id});
        std::push_heap(cand.begin(), cand.end(), FartherFirst{});
        res.push_back(Cand{d, id});
        std::push_heap(res.begin(), res.end(), CloserFirst{});
        if (res.size() > ef) {
          std::pop_heap(res.begin(), res.end(), CloserFirst{});
          res.pop_back();
        }
      }
    }
  }
}

/// Alg. 4 without extension / pruned-keeping: scan `sorted` by distance and
/// keep e unless some kept r is closer to e than e is to the base.
void heuristic(const Index::Impl& im, const std::vector<Cand>& sorted, std::size_t m, std::vector<Cand>& out) {
  out.clear();
  for (const Cand& e : sorted) {
    if (out.size() >= m) break;
    const float* ev = im.vec(e.id);
    bool keep = true;
    for (const Cand& r : out) {
      if (im.dist(ev, im.vec(r.id)) < e.dist) {
        keep = false;
        break;
      }
    }
    if (keep) out.push_back(e);
  }
}

/// Write id's list on `level` and add reverse edges, re-pruning full lists
/// (Alg. 1 lines 11-16; index.cpp:145-201).
void wire(Index::Impl& im, uint32_t id, int level, const std::vector<Cand>& chosen) {
  const std::size_t cap = im.degree_cap(level);
  std::vector<Cand> pool, kept;
  {
    std::lock_guard<std::mutex> g(im.lock_of(id));
    uint32_t* l = im.list(id, level);
    if (l[0] == 0) {
      l[0] = static_cast<uint32_t>(chosen.size());
      for (std::size_t i = 0; i < chosen.size(); ++i) l[1 + i] = chosen[i].id;
    } else {
      // a concurrent inserter linked to us first: merge, never overwrite
      const float* q = im.vec(id);
      pool.assign(chosen.begin(), chosen.end());
      for (uint32_t j = 0; j < l[0]; ++j) {
        const uint32_t e = l[1 + j];
        bool seen = false;
        for (const Cand& c : pool) seen = seen || c.id == e;
        if (!seen) pool.push_back(Cand{im.dist(q, im.vec(e)), e});
      }
      std::sort(pool.begin(), pool.end(), CloserFirst{});
      if (pool.size() > cap) {
        heuristic(im, pool, cap, kept);
        pool.swap(kept);
      }
      l[0] = static_cast<uint32_t>(pool.size());
      for (std::size_t i = 0; i < pool.size(); ++i) l[1 + i] = pool[i].id;
    }
  }
  for (const Cand& nb : chosen) {
    std::lock_guard<std::mutex> g(im.lock_of(nb.id));
    uint32_t* l = im.list(nb.id, level);
    const uint32_t n = l[0];
    bool present = false;
    for (uint32_t j = 0; j < n; ++j) present = present || l[1 + j] == id;
    if (present) continue;
    if (n < cap) {
      l[1 + n] = id;
      l[0] = n + 1;
      continue;
    }
    const float* nv = im.vec(nb.id);
    pool.clear();
    pool.push_back(Cand{nb.dist, id});
    for (uint32_t j = 0; j < n; ++j) pool.push_back(Cand{im.dist(nv, im.vec(l[1 + j])), l[1 + j]});
    std::sort(pool.begin(), pool.end(), CloserFirst{});
    heuristic(im, pool, cap, kept);
    l[0] = static_cast<uint32_t>(kept.size());
    for (std::size_t j = 0; j < kept.size(); ++j) l[1 + j] = kept[j].id;
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// Impl
// ---------------------------------------------------------------------------

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

int Index::Impl::draw_level() {
  const double u = 1.0 - static_cast<double>(splitmix64(rng_state) >> 11) * 0x1.0p-53;  // (0, 1]
  const double lvl = std::floor(-std::log(u) * mL);
  return static_cast<int>(std::min(lvl, static_cast<double>(gb::kMaxLevel)));
}

uint32_t Index::Impl::append(const float* v, uint64_t label) {
  const auto id = static_cast<uint32_t>(count);
  prepare(params.metric, v, vec_store.data() + std::size_t{id} * padded_dim, dim);
  label_store[id] = label;
  const int level = draw_level();
  level_store[id] = static_cast<uint8_t>(level);
  if (level > 0) {
    upper_offset[id] = upper_used;
    upper_used += static_cast<std::size_t>(level) * upper_stride;
    if (upper_store.size() < upper_used) {
      upper_store.resize(std::max(upper_used, upper_store.size() * 2), 0u);
      upper = upper_store.data();
    }
  }
  list0(id)[0] = 0;
  label_to_id.emplace(label, id);
  ++count;
  return id;
}

std::unique_ptr<gb::BuildScratch> Index::Impl::take_scratch() {
  std::lock_guard<std::mutex> g(scratch_mutex);
  if (scratch_free.empty()) return std::make_unique<gb::BuildScratch>();
  auto s = std::move(scratch_free.back());
  scratch_free.pop_back();
  return s;
}

void Index::Impl::give_scratch(std::unique_ptr<gb::BuildScratch> s) {
  std::lock_guard<std::mutex> g(scratch_mutex);
  scratch_free.push_back(std::move(s));
}

void Index::Impl::link(uint32_t id) {
  const int level = levels[id];
  const float* q = vec(id);
  std::unique_lock<std::mutex> top(top_mutex);
  const uint32_t ep = entry_point;
  const int top_level = max_level;
  if (ep == gb::kNoNode) {
    entry_point = id;
    max_level = level;
    return;
  }
  if (level <= top_level) top.unlock();  // only a new top node keeps the lock
  auto s = take_scratch();
  Cand cur{dist(q, vec(ep)), ep};
  for (int lc = top_level; lc > level; --lc) cur = descend(*this, q, cur, lc, s->nbuf);
  std::vector<Cand> eps{cur}, w, chosen;
  for (int lc = std::min(level, top_level); lc >= 0; --lc) {
    beam(*this, q, eps, ef_construction, lc, *s);
    w.assign(s->res.begin(), s->res.end());
    std::sort(w.begin(), w.end(), CloserFirst{});
    w.erase(std::remove_if(w.begin(), w.end(), [id](const Cand& c) { return c.id == id; }), w.end());
    heuristic(*this, w, M, chosen);
    wire(*this, id, lc, chosen);
    eps.swap(w);
  }
  give_scratch(std::move(s));
  if (level > top_level) {
    entry_point = id;
    max_level = level;
  }
}

// ---------------------------------------------------------------------------
// public construction / mutation API
// ---------------------------------------------------------------------------

Index::Index(const Params& params) : impl_(std::make_unique<Impl>(params)) {}
Index::Index(std::unique_ptr<Impl> impl) : impl_(std::move(impl)) {}
Index::~Index() = default;
Index::Index(Index&&) noexcept = default;
Index& Index::operator=(Index&&) noexcept = default;

void Index::add(const float* vec, uint64_t label) { add_batch(vec, &label, 1, 1); }

void Index::add_batch(const float* vecs, const uint64_t* labels, std::size_t n, std::size_t num_threads) {
  if (n == 0) return;
  if (vecs == nullptr || labels == nullptr) throw std::invalid_argument("add_batch: null input");
  std::unique_lock<std::shared_mutex> lk(impl_->api_mutex);
  Impl& im = *impl_;
  if (im.read_only) throw std::runtime_error("index is read-only (memory-mapped); load without mmap to modify");
  if (n > 1) {
    std::unordered_set<uint64_t> seen;
    seen.reserve(n);
    for (std::size_t i = 0; i < n; ++i)
      if (!seen.insert(labels[i]).second)
        throw std::invalid_argument("add_batch: duplicate label " + std::to_string(labels[i]) + " in batch");
  }
  for (std::size_t i = 0; i < n; ++i)
    if (im.label_to_id.count(labels[i]) != 0)
      throw std::invalid_argument("add: label " + std::to_string(labels[i]) + " already exists");
  const std::size_t need = im.count + n;
  if (need > im.capacity) {
    if (im.params.max_elements > 0)
      throw std::runtime_error("Index is full (max_elements = " + std::to_string(im.params.max_elements) + ")");
    im.grow(std::max({need, im.capacity * 2, std::size_t{1024}}));
  }
  im.label_to_id.reserve(im.count + n);
  const auto first = static_cast<uint32_t>(im.count);
  for (std::size_t i = 0; i < n; ++i) im.append(vecs + i * im.dim, labels[i]);
  parallel_range(n, num_threads, [&](std::size_t i) { im.link(first + static_cast<uint32_t>(i)); });
  std::lock_guard<std::mutex> g(im.dev_mutex);
  im.dev_stale = true;
}

void Index::mark_deleted(uint64_t label) {
  std::unique_lock<std::shared_mutex> lk(impl_->api_mutex);
  Impl& im = *impl_;
  auto it = im.label_to_id.find(label);
  if (it == im.label_to_id.end()) throw std::invalid_argument("mark_deleted: unknown label " + std::to_string(label));
  if (im.deleted[it->second] == 0) {
    im.deleted[it->second] = 1;
    ++im.num_deleted;
    std::lock_guard<std::mutex> g(im.dev_mutex);
    if (im.dev && !im.dev_stale && hgd_graph_set_deleted(im.dev, it->second, 1) != HGD_OK)
      throw std::runtime_error(std::string("mark_deleted: ") + hgd_last_error());
  }
}

bool Index::is_deleted(uint64_t label) const {
  std::shared_lock<std::shared_mutex> lk(impl_->api_mutex);
  auto it = impl_->label_to_id.find(label);
  return it != impl_->label_to_id.end() && impl_->deleted[it->second] != 0;
}

bool Index::contains(uint64_t label) const {
  std::shared_lock<std::shared_mutex> lk(impl_->api_mutex);
  return impl_->label_to_id.count(label) != 0;
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
  return im.count * (im.padded_dim * sizeof(float) + im.l0_stride * sizeof(uint32_t) + sizeof(uint64_t) * 2 + 2) +
         im.upper_used * sizeof(uint32_t);
}

std::vector<float> Index::get_vector(uint64_t label) const {
  std::shared_lock<std::shared_mutex> lk(impl_->api_mutex);
  auto it = impl_->label_to_id.find(label);
  if (it == impl_->label_to_id.end()) throw std::invalid_argument("get_vector: unknown label");
  const float* v = impl_->vec(it->second);
  return std::vector<float>(v, v + impl_->dim);
}

namespace tuning {
namespace {
std::atomic<bool> g_prefetch{true};
}
void set_prefetch(bool enabled) noexcept { g_prefetch.store(enabled); }
bool prefetch_enabled() noexcept { return g_prefetch.load(); }
}  // namespace tuning

}  // namespace hnsw
