// capi.cpp -- the hg_* C ABI (include/hnswgpu.h) over hnsw::Index.
// Exceptions never cross the boundary: each is mapped to a status code and
// its message kept for hg_last_error().
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "graph.hpp"
#include "hnsw/index.hpp"
#include "hnswgpu.h"

namespace hg {
// device_graph.cu: batch over a mirrored graph with scratch from a static device array
int search_noalloc(hgd_graph* g, const float* d_queries, uint64_t nq, uint32_t k, uint32_t ef, uint32_t ef_default,
                   void* d_out, void* stream);
}  // namespace hg

struct hg_index {
  hnsw::Index index;
};
struct hg_bruteforce {
  hnsw::BruteForceIndex bf;
};

namespace {

thread_local std::string g_msg;

template <typename Fn>
int guarded(Fn&& fn) {
  try {
    fn();
    return HG_OK;
  } catch (const std::invalid_argument& e) {
    g_msg = e.what();
    return HG_EINVAL;
  } catch (const std::out_of_range& e) {
    g_msg = e.what();
    return HG_ERANGE;
  } catch (const std::exception& e) {
    g_msg = e.what();
    return HG_ERUNTIME;
  } catch (...) {
    g_msg = "unknown error";
    return HG_ERUNTIME;
  }
}

struct PredicateFilter final : hnsw::Filter {
  int (*fn)(uint64_t, void*);
  void* ctx;
  bool allowed(uint64_t label) const override { return fn(label, ctx) != 0; }
};

/// hg_filter -> hnsw::Filter (owned by `keep`).
const hnsw::Filter* make_filter(const hg_filter* f, std::vector<std::unique_ptr<hnsw::Filter>>& keep) {
  if (f == nullptr || f->kind == HG_FILTER_NONE) return nullptr;
  if (f->kind == HG_FILTER_BITSET) {
    if (f->num_labels && !f->words) throw std::invalid_argument("filter: null bitset words");
    auto b = std::make_unique<hnsw::BitsetFilter>(f->num_labels);
    for (uint64_t w = 0; w < (f->num_labels + 63) / 64; ++w) {
      uint64_t bits = f->words[w];
      while (bits) {
        const uint64_t l = w * 64 + static_cast<uint64_t>(__builtin_ctzll(bits));
        bits &= bits - 1;
        if (l < f->num_labels) b->set(l);
      }
    }
    keep.push_back(std::move(b));
    return keep.back().get();
  }
  if (f->kind == HG_FILTER_PREDICATE) {
    if (!f->fn) throw std::invalid_argument("filter: null predicate");
    auto p = std::make_unique<PredicateFilter>();
    p->fn = f->fn;
    p->ctx = f->ctx;
    keep.push_back(std::move(p));
    return keep.back().get();
  }
  throw std::invalid_argument("filter: unknown kind");
}

hnsw::Metric metric_of(int m) {
  switch (m) {
    case HG_METRIC_L2: return hnsw::Metric::L2;
    case HG_METRIC_IP: return hnsw::Metric::InnerProduct;
    case HG_METRIC_COSINE: return hnsw::Metric::Cosine;
  }
  throw std::invalid_argument("unknown metric");
}

}  // namespace

extern "C" {

const char* hg_last_error(void) { return g_msg.c_str(); }

int hg_index_create(size_t dim, int metric, size_t M, size_t ef_construction, size_t max_elements, uint64_t seed,
                    hg_index** out) {
  return guarded([&] {
    if (!out) throw std::invalid_argument("hg_index_create: null out");
    hnsw::Params p;
    p.dim = dim;
    p.metric = metric_of(metric);
    p.M = M;
    p.ef_construction = ef_construction;
    p.max_elements = max_elements;
    p.seed = seed;
    *out = new hg_index{hnsw::Index(p)};
  });
}

int hg_index_load(const char* path, int mmap, hg_index** out) {
  return guarded([&] {
    if (!path || !out) throw std::invalid_argument("hg_index_load: null argument");
    *out = new hg_index{hnsw::Index::load(path, mmap != 0)};
  });
}

int hg_index_load_device(const char* path, int mmap, int device, hg_index** out) {
  return guarded([&] {
    if (!path || !out) throw std::invalid_argument("hg_index_load_device: null argument");
    *out = new hg_index{hnsw::Index::load_to_device(path, device, mmap != 0)};
  });
}

int hg_index_save(const hg_index* idx, const char* path) {
  return guarded([&] {
    if (!idx || !path) throw std::invalid_argument("hg_index_save: null argument");
    idx->index.save(path);
  });
}

void hg_index_free(hg_index* idx) { delete idx; }

int hg_index_add_batch(hg_index* idx, const float* vecs, const uint64_t* labels, size_t n, size_t num_threads) {
  return guarded([&] {
    if (!idx) throw std::invalid_argument("add_batch: null index");
    idx->index.add_batch(vecs, labels, n, num_threads);
  });
}

int hg_index_add_batch_gpu(hg_index* idx, const float* vecs, const uint64_t* labels, size_t n,
                           hg_build_options* opt) {
  return guarded([&] {
    if (!idx) throw std::invalid_argument("add_batch: null index");
    hnsw::GpuBuildOptions o;
    if (opt) {
      o.device = opt->device;
      o.wave_fraction = opt->wave_fraction;
      o.wave_min = opt->wave_min;
      o.wave_max = opt->wave_max;
      o.peers = opt->peers != 0;
    }
    const hnsw::GpuBuildStats st = idx->index.add_batch_gpu(vecs, labels, n, o);
    if (opt) {
      opt->waves = st.waves;
      opt->dropped_proposals = st.dropped_proposals;
      opt->seconds = st.seconds;
    }
  });
}

int hg_index_search(const hg_index* idx, const float* q, size_t k, size_t ef, const hg_filter* filter,
                    hg_neighbor* out, size_t* n_out) {
  return guarded([&] {
    if (!idx || !out || !n_out) throw std::invalid_argument("search: null pointer");
    std::vector<std::unique_ptr<hnsw::Filter>> keep;
    const auto res = idx->index.search(q, k, ef, make_filter(filter, keep));
    for (size_t i = 0; i < res.size(); ++i) out[i] = hg_neighbor{res[i].label, res[i].distance, 0};
    *n_out = res.size();
  });
}

int hg_index_search_batch(const hg_index* idx, const float* qs, size_t nq, size_t k, size_t ef, hg_neighbor* out,
                          size_t num_threads, const hg_filter* filter) {
  return guarded([&] {
    if (!idx) throw std::invalid_argument("search_batch: null index");
    std::vector<std::unique_ptr<hnsw::Filter>> keep;
    idx->index.search_batch(qs, nq, k, ef, reinterpret_cast<hnsw::Neighbor*>(out), num_threads,
                            make_filter(filter, keep));
  });
}

int hg_index_search_batch_ex(const hg_index* idx, const float* qs, size_t nq, size_t k, size_t ef,
                             hg_neighbor* out, const hg_batch_options* o) {
  return guarded([&] {
    if (!idx) throw std::invalid_argument("search_batch: null index");
    hnsw::SearchOptions opt;
    std::vector<std::unique_ptr<hnsw::Filter>> keep;
    std::vector<const hnsw::Filter*> table;
    if (o) {
      opt.ef_per_query = o->ef_per_query;
      opt.k_per_query = o->k_per_query;
      for (size_t i = 0; i < o->num_filters; ++i) {
        const hnsw::Filter* f = make_filter(&o->filters[i], keep);
        if (!f) throw std::invalid_argument("search_batch: empty filter in table");
        table.push_back(f);
      }
      opt.filters = table.empty() ? nullptr : table.data();
      opt.num_filters = table.size();
      opt.filter_of_query = o->filter_of_query;
      opt.stream = o->stream;
      opt.precision = o->precision;
      opt.counters = o->counters;
      opt.hash_slots = o->hash_slots;
      opt.cand_cap = o->cand_cap;
      opt.warps_per_block = o->warps_per_block;
      opt.pool_cap = o->pool_cap;
      opt.queries_on_device = o->queries_on_device != 0;
      opt.out_on_device = o->out_on_device != 0;
      opt.use_graph = o->use_graph != 0;
      opt.filter_scan_permille = o->filter_scan_permille;
      opt.rerank_factor = o->rerank_factor;
      opt.warps_per_query = o->warps_per_query;
      opt.lists_per_step = o->lists_per_step;
      opt.filter_scan_mode = o->filter_scan_mode;
    }
    idx->index.search_batch_ex(qs, nq, k, ef, reinterpret_cast<hnsw::Neighbor*>(out), opt);
  });
}

int hg_index_autotune(hg_index* idx, const float* qs, size_t nq, size_t k, size_t ef_max, int precision,
                      const uint32_t* ef_per_query, char* json, size_t json_cap, size_t* json_len) {
  return guarded([&] {
    if (!idx || !qs) throw std::invalid_argument("autotune: null pointer");
    const std::string out =
        hnsw::gb::autotune(*idx->index.impl(), qs, nq, static_cast<uint32_t>(k),
                           static_cast<uint32_t>(std::min<size_t>(ef_max, 1024)), precision, ef_per_query);
    if (json_len) *json_len = out.size() + 1;
    if (json && json_cap) {
      const size_t m = std::min(json_cap - 1, out.size());
      std::memcpy(json, out.data(), m);
      json[m] = 0;
    }
  });
}

int hg_index_set_tuning(hg_index* idx, const char* json) {
  return guarded([&] {
    if (!idx || !json) throw std::invalid_argument("set_tuning: null pointer");
    hnsw::gb::apply_tuning_json(*idx->index.impl(), json);
  });
}

int hg_index_mark_deleted(hg_index* idx, uint64_t label) {
  return guarded([&] {
    if (!idx) throw std::invalid_argument("mark_deleted: null index");
    idx->index.mark_deleted(label);
  });
}

int hg_index_is_deleted(const hg_index* idx, uint64_t label, int* out) {
  return guarded([&] {
    if (!idx || !out) throw std::invalid_argument("is_deleted: null pointer");
    *out = idx->index.is_deleted(label) ? 1 : 0;
  });
}

int hg_index_contains(const hg_index* idx, uint64_t label, int* out) {
  return guarded([&] {
    if (!idx || !out) throw std::invalid_argument("contains: null pointer");
    *out = idx->index.contains(label) ? 1 : 0;
  });
}

int hg_index_get_vector(const hg_index* idx, uint64_t label, float* out, size_t dim) {
  return guarded([&] {
    if (!idx || !out) throw std::invalid_argument("get_vector: null pointer");
    const auto v = idx->index.get_vector(label);
    if (dim < v.size()) throw std::invalid_argument("get_vector: buffer too small");
    std::memcpy(out, v.data(), v.size() * sizeof(float));
  });
}

int hg_index_set_ef(hg_index* idx, size_t ef) {
  return guarded([&] {
    if (!idx) throw std::invalid_argument("set_ef: null index");
    idx->index.set_ef(ef);
  });
}

int hg_index_set_device(hg_index* idx, int device) {
  return guarded([&] {
    if (!idx) throw std::invalid_argument("set_device: null index");
    idx->index.set_device(device);
  });
}

size_t hg_index_size(const hg_index* idx) { return idx ? idx->index.size() : 0; }
size_t hg_index_dim(const hg_index* idx) { return idx ? idx->index.dim() : 0; }
int hg_index_metric(const hg_index* idx) { return idx ? static_cast<int>(idx->index.metric()) : -1; }
size_t hg_index_M(const hg_index* idx) { return idx ? idx->index.params().M : 0; }
size_t hg_index_ef_construction(const hg_index* idx) { return idx ? idx->index.params().ef_construction : 0; }
size_t hg_index_ef(const hg_index* idx) { return idx ? idx->index.ef() : 0; }
size_t hg_index_capacity(const hg_index* idx) { return idx ? idx->index.capacity() : 0; }
int hg_index_max_level(const hg_index* idx) { return idx ? idx->index.max_level() : -1; }
int hg_index_read_only(const hg_index* idx) { return idx && idx->index.read_only() ? 1 : 0; }
size_t hg_index_memory_usage(const hg_index* idx) { return idx ? idx->index.memory_usage() : 0; }

int hg_bruteforce_create(size_t dim, int metric, hg_bruteforce** out) {
  return guarded([&] {
    if (!out) throw std::invalid_argument("bruteforce: null out");
    *out = new hg_bruteforce{hnsw::BruteForceIndex(dim, metric_of(metric))};
  });
}

int hg_bruteforce_add(hg_bruteforce* bf, const float* vecs, const uint64_t* labels, size_t n) {
  return guarded([&] {
    if (!bf || (n && !vecs)) throw std::invalid_argument("bruteforce add: null pointer");
    bf->bf.add(vecs, labels, n);
  });
}

int hg_bruteforce_search_batch(const hg_bruteforce* bf, const float* qs, size_t nq, size_t k, hg_neighbor* out,
                               const hg_filter* filter) {
  return guarded([&] {
    if (!bf) throw std::invalid_argument("bruteforce search: null index");
    std::vector<std::unique_ptr<hnsw::Filter>> keep;
    bf->bf.search_batch(qs, nq, k, reinterpret_cast<hnsw::Neighbor*>(out), 0, make_filter(filter, keep));
  });
}

void hg_bruteforce_free(hg_bruteforce* bf) { delete bf; }

int hg_bruteforce_set_path(hg_bruteforce* bf, int path) {
  return guarded([&] {
    if (!bf) throw std::invalid_argument("bruteforce: null index");
    bf->bf.set_gpu_path(path);
  });
}

int hg_bruteforce_last_path(const hg_bruteforce* bf) { return bf ? bf->bf.last_gpu_path() : 0; }

struct hg_server {
  hnsw::gb::Server* s;
};

int hg_server_create(const hg_index* idx, const hg_server_config* cfg, hg_server** out) {
  return guarded([&] {
    if (!idx || !out) throw std::invalid_argument("server: null argument");
    hg_server_config c{};
    if (cfg) c = *cfg;
    *out = new hg_server{hnsw::gb::server_new(*idx->index.impl(), c)};
  });
}

int hg_server_submit(hg_server* s, const hg_request* r, uint64_t* ticket) {
  return guarded([&] {
    if (!s || !r || !ticket) throw std::invalid_argument("server submit: null argument");
    *ticket = hnsw::gb::server_submit(s->s, *r);
  });
}

int hg_server_wait(hg_server* s, uint64_t ticket, double* latency_ms) {
  return guarded([&] {
    if (!s) throw std::invalid_argument("server wait: null server");
    hnsw::gb::server_wait(s->s, ticket, latency_ms);
  });
}

int hg_server_replay(hg_server* s, const hg_request* reqs, const double* arrival_s, size_t n,
                     hg_server_stats* stats) {
  return hg_server_replay_latencies(s, reqs, arrival_s, n, stats, nullptr);
}

int hg_server_replay_latencies(hg_server* s, const hg_request* reqs, const double* arrival_s, size_t n,
                               hg_server_stats* stats, double* latency_ms) {
  return guarded([&] {
    if (!s || (n && (!reqs || !arrival_s)) || !stats) throw std::invalid_argument("server replay: null argument");
    hnsw::gb::server_replay(s->s, reqs, arrival_s, n, stats, latency_ms);
  });
}

int hg_server_stats_get(hg_server* s, hg_server_stats* out) {
  return guarded([&] {
    if (!s || !out) throw std::invalid_argument("server stats: null argument");
    hnsw::gb::server_stats(s->s, out);
  });
}

void hg_server_destroy(hg_server* s) {
  if (s) hnsw::gb::server_delete(s->s);
  delete s;
}

int hg_index_search_batch_noalloc(const hg_index* idx, const float* queries, size_t nq, size_t k, size_t ef,
                                  hg_neighbor* out, void* stream) {
  return guarded([&] {
    if (!idx) throw std::invalid_argument("search_batch (no-alloc): null index");
    if (k == 0) throw std::invalid_argument("search_batch: k must be > 0");
    if (k > 0xFFFFFFFFull || ef > 0xFFFFFFFFull) throw std::invalid_argument("search_batch: k / ef out of range");
    const hnsw::Index::Impl* im = idx->index.impl();
    std::shared_lock<std::shared_mutex> lk(im->api_mutex);
    hgd_graph* g = nullptr;
    {
      std::lock_guard<std::mutex> dg(im->dev_mutex);
      if (im->dev == nullptr || im->dev_stale)
        throw std::runtime_error(
            "search_batch (no-alloc): the graph is not mirrored on the GPU; run one allocating search first");
      g = im->dev;
    }
    const uint32_t ef_default = static_cast<uint32_t>(std::min<size_t>(im->ef_search, 0xFFFFFFFFull));
    const int rc = hg::search_noalloc(g, queries, nq, static_cast<uint32_t>(k), static_cast<uint32_t>(ef),
                                      ef_default, out, stream);
    if (rc == HGD_EINVAL) throw std::invalid_argument(hgd_last_error());
    if (rc != HGD_OK) throw std::runtime_error(hgd_last_error());
  });
}

int hg_set_distance_order(int order) {
  return guarded([&] {
    if (order < HG_ORDER_SCALAR || order > HG_ORDER_NEON) throw std::invalid_argument("unknown distance order");
    hnsw::simd::set_active(static_cast<hnsw::simd::Isa>(order));
  });
}

int hg_get_distance_order(void) { return static_cast<int>(hnsw::simd::active().isa); }

}  // extern "C"
