// build.cpp -- CPU graph construction behind hnsw::Index::add / add_batch.
//
// The search kernels walk the graph the reference builds, so this builder
// produces that graph: Malkov & Yashunin's insertion (Alg. 1) with the
// neighbour-selection heuristic (Alg. 4, no candidate extension, no kept
// pruned connections), as the reference's src/index.cpp:94-306 and its
// locked layer search src/search_layer.cpp:29-134 define it.  What has to be
// the same for the same graph:
//   * levels: splitmix64 draws from the seed in input order, u in (0, 1]
//     from the top 53 bits, level = floor(-ln(u) / ln M), at most 64;
//   * the layer search's order and rules: candidates by (distance, internal
//     id), a candidate accepted while the result set holds fewer than ef or
//     it is strictly closer than the farthest result, the search ending when
//     the closest open candidate is farther than the farthest of ef results;
//   * M neighbours chosen per layer (level 0 included), reverse edges
//     appended while a list has room and re-chosen by Alg. 4 from the old
//     list plus the new node when it is full (cap 2M at level 0, M above);
//   * upper-layer blocks laid out in input order.
// With one thread the saved file is byte for byte the reference's (tested);
// with more threads, as there, the graph depends on thread timing.
//
// Design.  insert_batch stores the batch first -- vectors prepared, every
// level drawn and every upper block placed, with one exact resize -- and
// then workers pull node ids from a shared counter, each with its own
// Inserter: visited stamps, a candidate heap and a result list kept sorted,
// and the buffers of one insertion.  Lists are read and written under the
// node's stripe lock; the entry point and top level under top_mutex, held
// for a whole insertion only by a node that becomes the new top.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <exception>
#include <functional>
#include <queue>
#include <stdexcept>
#include <string>
#include <thread>

#include "graph.hpp"

namespace hnsw::gb {
namespace {

// one splitmix64 step (the reference's level source, src/index.cpp:20-28)
uint64_t mix_next(uint64_t& state) noexcept {
  uint64_t z = (state += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

// the level of a node from one draw: u = 1 - (draw >> 11) 2^-53 in (0, 1]
int level_from(uint64_t draw, double mL) {
  const double u = 1.0 - std::ldexp(static_cast<double>(draw >> 11), -53);
  const double l = std::floor(-std::log(u) * mL);
  return l >= kMaxLevel ? kMaxLevel : static_cast<int>(l);
}

// space.hpp:31-40: a copy, or for cosine the unit vector with the norm
// accumulated in double in element order
void prepare_row(Metric m, const float* src, float* dst, std::size_t dim) {
  if (m != Metric::Cosine) {
    std::copy(src, src + dim, dst);
    return;
  }
  double ss = 0.0;
  for (std::size_t i = 0; i < dim; ++i) ss += static_cast<double>(src[i]) * src[i];
  const float scale = ss > 0.0 ? static_cast<float>(1.0 / std::sqrt(ss)) : 1.0f;
  for (std::size_t i = 0; i < dim; ++i) dst[i] = src[i] * scale;
}

class Inserter {
 public:
  explicit Inserter(Index::Impl& g) : g_(g), stamp_(g.capacity, 0u) {}

  // Alg. 1 for node id, whose vector and level are stored already
  void run(uint32_t id) {
    const int level = g_.levels[id];
    const float* q = g_.vec(id);
    std::unique_lock<std::mutex> top(g_.top_mutex);
    const uint32_t ep = g_.entry_point;
    const int top_level = g_.max_level;
    if (ep == kNoNode) {  // the first node
      g_.entry_point = id;
      g_.max_level = level;
      return;
    }
    if (level <= top_level) top.unlock();
    Cand at{dist_to(q, ep), ep};
    for (int lc = top_level; lc > level; --lc) at = greedy(q, at, lc);
    entries_.assign(1, at);
    for (int lc = std::min(level, top_level); lc >= 0; --lc) {
      layer_search(q, lc);
      found_.erase(std::remove_if(found_.begin(), found_.end(), [id](const Cand& c) { return c.id == id; }),
                   found_.end());
      select(found_, g_.M, chosen_);
      link_forward(id, lc);
      link_backward(id, lc);
      entries_.swap(found_);
    }
    if (level > top_level) {  // still holding top_mutex
      g_.entry_point = id;
      g_.max_level = level;
    }
  }

 private:
  float dist_to(const float* q, uint32_t id) const { return g_.dist(q, g_.vec(id)); }

  // a copy of node's list at level, taken under its lock
  void read_list(uint32_t node, int level) {
    std::lock_guard<std::mutex> g(g_.lock_of(node));
    const uint32_t* l = g_.list(node, level);
    nbrs_.assign(l + 1, l + 1 + l[0]);
  }

  // greedy descent: the first strictly closer neighbour in list order moves
  // the walk, until a pass over the list moves nothing
  Cand greedy(const float* q, Cand at, int level) {
    bool moved = true;
    while (moved) {
      moved = false;
      read_list(at.id, level);
      for (uint32_t nb : nbrs_) {
        const float d = dist_to(q, nb);
        if (d < at.dist) {
          at = Cand{d, nb};
          moved = true;
        }
      }
    }
    return at;
  }

  void next_stamp() {
    if (stamp_.size() < g_.capacity) stamp_.resize(g_.capacity, 0u);
    if (++stamp_id_ == 0) {  // wrapped: every old stamp must read as unvisited
      std::fill(stamp_.begin(), stamp_.end(), 0u);
      stamp_id_ = 1;
    }
  }
  bool seen(uint32_t id) {
    if (stamp_[id] == stamp_id_) return true;
    stamp_[id] = stamp_id_;
    return false;
  }

  // keep found_ sorted by (distance, id) with at most ef entries
  void offer(const Cand& c, std::size_t ef) {
    found_.insert(std::upper_bound(found_.begin(), found_.end(), c, closer), c);
    if (found_.size() > ef) found_.pop_back();
  }

  // Alg. 2 (unfiltered) from entries_ on one layer; found_ ends sorted
  void layer_search(const float* q, int level) {
    const std::size_t ef = g_.ef_construction;
    next_stamp();
    found_.clear();
    open_ = {};
    for (const Cand& e : entries_) {
      if (seen(e.id)) continue;
      open_.push(e);
      offer(e, ef);
    }
    while (!open_.empty()) {
      const Cand c = open_.top();
      if (found_.size() >= ef && c.dist > found_.back().dist) break;
      open_.pop();
      read_list(c.id, level);
      for (uint32_t nb : nbrs_) {
        if (seen(nb)) continue;
        const float d = dist_to(q, nb);
        if (found_.size() < ef || d < found_.back().dist) {
          open_.push(Cand{d, nb});
          offer(Cand{d, nb}, ef);
        }
      }
    }
  }

  // Alg. 4: from candidates sorted by (distance, id), keep one unless a kept
  // neighbour is strictly closer to it than the base node is
  void select(const std::vector<Cand>& sorted, std::size_t m, std::vector<Cand>& out) const {
    out.clear();
    for (const Cand& c : sorted) {
      if (out.size() >= m) break;
      const float* cv = g_.vec(c.id);
      const bool dominated =
          std::any_of(out.begin(), out.end(), [&](const Cand& k) { return g_.dist(cv, g_.vec(k.id)) < c.dist; });
      if (!dominated) out.push_back(c);
    }
  }

  // the node's own list: the chosen neighbours, merged with edges that a
  // concurrent insertion added first (parallel builds) and re-chosen if full
  void link_forward(uint32_t id, int level) {
    const std::size_t cap = g_.degree_cap(level);
    std::lock_guard<std::mutex> g(g_.lock_of(id));
    uint32_t* l = g_.list(id, level);
    if (l[0] != 0) {
      const float* q = g_.vec(id);
      pool_.assign(chosen_.begin(), chosen_.end());
      for (uint32_t j = 1; j <= l[0]; ++j) {
        const uint32_t e = l[j];
        if (std::none_of(pool_.begin(), pool_.end(), [e](const Cand& c) { return c.id == e; }))
          pool_.push_back(Cand{dist_to(q, e), e});
      }
      std::sort(pool_.begin(), pool_.end(), closer);
      if (pool_.size() > cap) {
        select(pool_, cap, kept_);
        pool_.swap(kept_);
      }
      write(l, pool_);
      return;
    }
    write(l, chosen_);
  }

  // reverse edges: appended while there is room, else the full list plus
  // the new node re-chosen by Alg. 4
  void link_backward(uint32_t id, int level) {
    const std::size_t cap = g_.degree_cap(level);
    for (const Cand& nb : chosen_) {
      std::lock_guard<std::mutex> g(g_.lock_of(nb.id));
      uint32_t* l = g_.list(nb.id, level);
      const uint32_t n = l[0];
      if (std::find(l + 1, l + 1 + n, id) != l + 1 + n) continue;
      if (n < cap) {
        l[1 + n] = id;
        l[0] = n + 1;
        continue;
      }
      const float* nv = g_.vec(nb.id);
      pool_.assign(1, Cand{nb.dist, id});
      for (uint32_t j = 1; j <= n; ++j) pool_.push_back(Cand{g_.dist(nv, g_.vec(l[j])), l[j]});
      std::sort(pool_.begin(), pool_.end(), closer);
      select(pool_, cap, kept_);
      write(l, kept_);
    }
  }

  static void write(uint32_t* l, const std::vector<Cand>& v) {
    l[0] = static_cast<uint32_t>(v.size());
    for (std::size_t i = 0; i < v.size(); ++i) l[1 + i] = v[i].id;
  }

  Index::Impl& g_;
  std::vector<uint32_t> stamp_;
  uint32_t stamp_id_ = 0;
  std::vector<uint32_t> nbrs_;
  std::vector<Cand> entries_, found_, chosen_, pool_, kept_;
  std::priority_queue<Cand, std::vector<Cand>, FartherFirst> open_;  // closest on top
};

// Store the batch: rows prepared, levels drawn in input order, upper blocks
// placed after the ones in use; returns the first new id.
uint32_t store_batch(Index::Impl& g, const float* vecs, const uint64_t* labels, std::size_t n) {
  const std::size_t need = g.count + n;
  if (need > g.capacity) {
    if (g.params.max_elements > 0)
      throw std::runtime_error("Index is full (max_elements = " + std::to_string(g.params.max_elements) + ")");
    g.grow(std::max<std::size_t>(need, g.capacity + g.capacity / 2 + 1024));
  }
  const auto first = static_cast<uint32_t>(g.count);
  std::size_t upper_need = g.upper_used;
  for (std::size_t i = 0; i < n; ++i) {
    const uint32_t id = first + static_cast<uint32_t>(i);
    const int level = level_from(mix_next(g.rng_state), g.mL);
    g.level_store[id] = static_cast<uint8_t>(level);
    if (level > 0) {
      g.upper_offset[id] = upper_need;
      upper_need += static_cast<std::size_t>(level) * g.upper_stride;
    }
  }
  if (upper_need > g.upper_store.size()) {
    g.upper_store.resize(upper_need, 0u);
    g.upper = g.upper_store.data();
  }
  g.upper_used = upper_need;
  g.label_to_id.reserve(need);
  for (std::size_t i = 0; i < n; ++i) {
    const uint32_t id = first + static_cast<uint32_t>(i);
    prepare_row(g.params.metric, vecs + i * g.dim, g.vec_store.data() + std::size_t{id} * g.padded_dim, g.dim);
    g.label_store[id] = labels[i];
    g.list0(id)[0] = 0;
    g.label_to_id.emplace(labels[i], id);
  }
  g.count = need;
  return first;
}

}  // namespace

void insert_batch(Index::Impl& g, const float* vecs, const uint64_t* labels, std::size_t n, std::size_t threads) {
  const uint32_t first = store_batch(g, vecs, labels, n);
  if (threads == 0) threads = std::max(1u, std::thread::hardware_concurrency());
  threads = std::min(threads, n);
  std::atomic<std::size_t> next{0};
  std::atomic<bool> stop{false};
  std::exception_ptr err;
  std::mutex err_mu;
  auto worker = [&]() {
    try {
      Inserter ins(g);
      for (std::size_t i = next++; i < n && !stop.load(std::memory_order_relaxed); i = next++)
        ins.run(first + static_cast<uint32_t>(i));
    } catch (...) {
      std::lock_guard<std::mutex> lk(err_mu);
      if (!err) err = std::current_exception();
      stop = true;
    }
  };
  std::vector<std::thread> pool;
  for (std::size_t t = 1; t < threads; ++t) pool.emplace_back(worker);
  worker();  // the calling thread works too
  for (auto& t : pool) t.join();
  if (err) std::rethrow_exception(err);
}

GpuBuildStats insert_batch_gpu(Index::Impl& g, const float* vecs, const uint64_t* labels, std::size_t n,
                               const GpuBuildOptions& opt) {
  // the GPU builder's limits, checked before the index changes
  if (g.count + n >= (std::size_t{1} << 24))
    throw std::invalid_argument("add_batch_gpu: the GPU builder takes fewer than 2^24 nodes");
  if (g.M > 32) throw std::invalid_argument("add_batch_gpu: the GPU builder takes M <= 32");
  if (g.padded_dim > 1024) throw std::invalid_argument("add_batch_gpu: the GPU builder takes dim <= 1024");
  if (g.ef_construction > 1024)
    throw std::invalid_argument("add_batch_gpu: the GPU builder takes ef_construction <= 1024");
  if (!(opt.wave_fraction >= 0.0)) throw std::invalid_argument("add_batch_gpu: wave_fraction must be >= 0");
  const std::size_t old_count = g.count, old_upper = g.upper_used;
  const uint64_t old_rng = g.rng_state;
  const uint32_t first = store_batch(g, vecs, labels, n);
  hgd_build_args a{};
  a.count = g.count;
  a.first = first;
  a.dim = g.dim;
  a.padded_dim = g.padded_dim;
  a.M = g.M;
  a.ef_construction = g.ef_construction;
  a.metric = static_cast<int32_t>(g.params.metric);
  a.max_level = g.max_level;
  a.entry_point = g.entry_point;
  a.wave_min = opt.wave_min;
  a.wave_max = opt.wave_max;
  a.wave_fraction = opt.wave_fraction;
  a.peers = opt.peers ? 1 : 0;
  a.vectors = g.vecs;
  a.level0 = g.l0;
  a.upper = g.upper;
  a.upper_words = g.upper_used;
  a.upper_offset = g.upper_offset.data();
  a.levels = g.levels;
  const auto t0 = std::chrono::steady_clock::now();
  const int rc = hgd_build_graph(&a, opt.device >= 0 ? opt.device : g.device);
  const auto t1 = std::chrono::steady_clock::now();
  if (rc != HGD_OK) {
    // undo the store: labels, count, upper blocks and the level draws
    const std::string msg = hgd_last_error();
    for (std::size_t i = old_count; i < g.count; ++i) {
      g.label_to_id.erase(g.label_store[i]);
      g.list0(static_cast<uint32_t>(i))[0] = 0;
    }
    std::fill(g.upper_store.begin() + static_cast<std::ptrdiff_t>(old_upper), g.upper_store.end(), 0u);
    g.count = old_count;
    g.upper_used = old_upper;
    g.rng_state = old_rng;
    if (rc == HGD_EINVAL) throw std::invalid_argument("add_batch_gpu: " + msg);
    throw std::runtime_error("add_batch_gpu: " + msg);
  }
  g.entry_point = a.entry_point;
  g.max_level = a.max_level;
  GpuBuildStats st;
  st.waves = a.waves;
  st.dropped_proposals = a.dropped_proposals;
  st.seconds = std::chrono::duration<double>(t1 - t0).count();
  return st;
}

}  // namespace hnsw::gb
