// server.cpp -- continuous-batching query server over one GPU index.
//
// Requests (a block of queries with their own k, ef and optional filter)
// wait in a FIFO.  A dispatcher thread admits them into a batch whenever one
// of `max_inflight` batch slots is free and the device-memory budget allows
// it, and enqueues the batch asynchronously on the slot's stream (its own
// workspace, so batches overlap on the GPU).  A completion thread polls the
// batches' events, copies each request's rows to its output and records the
// request's latency from arrival to completion.  The traversal itself is the
// same per-query algorithm as search_batch, so a request's answer does not
// depend on what it was batched with.  The kernels write each query's result
// row straight into mapped pinned host memory and then raise that query's
// done flag (system-scope fence first), so a request is returned as soon as
// its own queries are finished, not when the slowest query of its batch is.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <shared_mutex>
#include <stdexcept>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "graph.hpp"
#include "hnswgpu.h"

namespace hnsw::gb {

using Clock = std::chrono::steady_clock;

struct ServerRequest {
  const float* queries = nullptr;
  uint32_t nq = 0, k = 0, ef = 0;
  bool has_filter = false;
  FilterBits filter;
  hg_neighbor* out = nullptr;
  Clock::time_point arrival;
  double latency_ms = 0.0;
  bool done = false;
  int status = HG_OK;
  std::string error;
};

template <typename T>
struct Pinned {
  T* p = nullptr;
  T* dev = nullptr;  // device view of mapped memory
  size_t n = 0;
  bool ensure(size_t need, bool mapped = false) {
    if (need <= n) return true;
    if (p) cudaFreeHost(p);
    p = dev = nullptr;
    n = 0;
    if (cudaHostAlloc(reinterpret_cast<void**>(&p), need * sizeof(T),
                      mapped ? cudaHostAllocMapped : cudaHostAllocDefault) != cudaSuccess)
      return false;
    if (mapped && cudaHostGetDevicePointer(reinterpret_cast<void**>(&dev), p, 0) != cudaSuccess) {
      cudaFreeHost(p);
      p = nullptr;
      return false;
    }
    n = need;
    return true;
  }
  ~Pinned() {
    if (p) cudaFreeHost(p);
  }
};

struct BatchSlot {
  cudaStream_t stream = nullptr;
  cudaEvent_t ev = nullptr;
  Pinned<float> q;
  Pinned<hg_neighbor> out;  // mapped: the kernels write rows here
  Pinned<uint32_t> done;    // mapped: per-query done flags
  std::vector<char> req_done;
  size_t ndone = 0;
  std::vector<uint32_t> efq, kq;
  std::vector<int32_t> fsel;
  std::vector<hgd_bitset> ftab;
  std::vector<ServerRequest*> reqs;
  std::vector<uint32_t> offset;
  uint32_t kstride = 0;
  uint64_t bytes = 0;  // admitted device bytes
  bool inflight = false;
};

class Server {
 public:
  Server(const Index::Impl& im, const hg_server_config& cfg) : im_(im) {
    max_inflight_ = std::max<uint32_t>(1, std::min<uint32_t>(cfg.max_inflight ? cfg.max_inflight : 4, 15));
    max_batch_ = cfg.max_batch_queries ? cfg.max_batch_queries : 4096;
    precision_ = cfg.precision;
    filter_scan_permille_ = cfg.filter_scan_permille;
    rerank_factor_ = cfg.rerank_factor;
    warps_per_query_ = cfg.warps_per_query;
    lists_per_step_ = cfg.lists_per_step;
    filter_scan_mode_ = cfg.filter_scan_mode;
    {
      std::shared_lock<std::shared_mutex> lk(im.api_mutex);
      g_ = im.device_graph();
      dim_ = static_cast<uint32_t>(im.dim);
      ef_default_ = static_cast<uint32_t>(std::min<size_t>(im.ef_search, 0xFFFFFFFFu));
      n_ = im.count;
    }
    size_t free_b = 0, total_b = 0;
    cudaSetDevice(im.device);
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) throw std::runtime_error("server: cudaMemGetInfo failed");
    budget_ = cfg.memory_budget ? cfg.memory_budget : static_cast<uint64_t>(free_b * 0.5);
    slots_.resize(max_inflight_);
    for (auto& s : slots_) {
      if (cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking) != cudaSuccess ||
          cudaEventCreateWithFlags(&s.ev, cudaEventDisableTiming) != cudaSuccess)
        throw std::runtime_error("server: cannot create streams");
    }
    dispatcher_ = std::thread([this] { dispatch_loop(); });
    completer_ = std::thread([this] { complete_loop(); });
  }

  ~Server() {
    {
      std::lock_guard<std::mutex> lk(mu_);
      stop_ = true;
    }
    cv_.notify_all();
    cv_launched_.notify_all();
    dispatcher_.join();
    completer_.join();
    for (auto& s : slots_) {
      if (s.stream) cudaStreamDestroy(s.stream);
      if (s.ev) cudaEventDestroy(s.ev);
    }
  }

  uint64_t submit(const hg_request& r, Clock::time_point arrival) {
    if (!r.queries || !r.out) throw std::invalid_argument("server submit: null pointer");
    if (r.k == 0) throw std::invalid_argument("search_batch: k must be > 0");
    if (r.nq == 0) throw std::invalid_argument("server submit: empty request");
    auto q = std::make_unique<ServerRequest>();
    q->queries = r.queries;
    q->nq = r.nq;
    q->k = r.k;
    q->ef = r.ef;
    q->out = r.out;
    q->arrival = arrival;
    if (r.filter && r.filter->kind != HG_FILTER_NONE) {
      q->has_filter = true;
      if (r.filter->kind == HG_FILTER_BITSET) {
        q->filter.view.words = r.filter->words;
        q->filter.view.num_bits = r.filter->num_labels;
        q->filter.view.label_space = 1;
      } else if (r.filter->kind == HG_FILTER_PREDICATE && r.filter->fn) {
        q->filter.owned.assign((n_ + 63) / 64, 0);
        for (size_t i = 0; i < n_; ++i)
          if (r.filter->fn(im_.labels[i], r.filter->ctx)) q->filter.owned[i >> 6] |= 1ULL << (i & 63);
        q->filter.view.words = q->filter.owned.data();
        q->filter.view.num_bits = n_;
        q->filter.view.label_space = 0;
      } else {
        throw std::invalid_argument("server submit: unknown filter kind");
      }
    }
    std::lock_guard<std::mutex> lk(mu_);
    const uint64_t t = ++next_ticket_;
    ServerRequest* raw = q.get();
    reqs_.emplace(t, std::move(q));
    pending_.push_back(raw);
    cv_.notify_all();
    return t;
  }

  void wait(uint64_t t, double* latency_ms, int* status, std::string* err) {
    std::unique_lock<std::mutex> lk(mu_);
    auto it = reqs_.find(t);
    if (it == reqs_.end()) throw std::invalid_argument("server wait: unknown ticket");
    ServerRequest* r = it->second.get();
    cv_done_.wait(lk, [&] { return r->done; });
    if (latency_ms) *latency_ms = r->latency_ms;
    if (status) *status = r->status;
    if (err) *err = r->error;
    reqs_.erase(it);
  }

  void stats(hg_server_stats* s) {
    std::lock_guard<std::mutex> lk(mu_);
    std::memset(s, 0, sizeof(*s));
    s->requests = lat_.size();
    s->queries = queries_done_;
    s->batches = batches_;
    s->mean_batch_queries = batches_ ? static_cast<double>(batch_queries_) / batches_ : 0.0;
    s->memory_waits = memory_waits_;
    if (!lat_.empty()) {
      std::vector<double> v = lat_;
      std::sort(v.begin(), v.end());
      auto pct = [&](double p) {
        const size_t i = std::min(v.size() - 1, static_cast<size_t>(p * static_cast<double>(v.size())));
        return v[i];
      };
      s->p50_ms = pct(0.50);
      s->p99_ms = pct(0.99);
      s->p999_ms = pct(0.999);
      s->max_ms = v.back();
      double sum = 0;
      for (double x : v) sum += x;
      s->mean_ms = sum / static_cast<double>(v.size());
      s->elapsed_s = std::chrono::duration<double>(last_done_ - first_arrival_).count();
      s->qps = s->elapsed_s > 0 ? static_cast<double>(queries_done_) / s->elapsed_s : 0.0;
    }
  }

  void reset_stats() {
    std::lock_guard<std::mutex> lk(mu_);
    lat_.clear();
    queries_done_ = batches_ = batch_queries_ = memory_waits_ = 0;
    have_first_ = false;
  }

 private:
  // Device bytes one batch needs beyond the resident graph (an upper bound):
  // queries, per-query arrays and results, ef-bucket lists, rerank pools, the
  // two spill-pool tiers, visited bitmaps and the rerun pass's scratch.
  uint64_t batch_bytes(uint64_t nq, uint32_t kstride, uint32_t ef_max) const {
    const uint64_t per_q = uint64_t{dim_} * 4 + uint64_t{kstride} * 16 + 64 + 12 * 4 + 4 * ((ef_max + 31) / 32 * 32);
    const uint64_t pool = std::min<uint64_t>(1ull << 30, 152ull * 64 * std::min<uint64_t>(std::max<uint64_t>(n_, 1), 8192) * 8) +
                          (2ull << 30);
    const uint64_t bitmaps = std::min<uint64_t>(1ull << 30, 152ull * 64 * ((n_ + 31) / 32 + 1) * 4);
    const uint64_t rerun = 32ull * (std::max<uint64_t>(n_, 1) * 8 + ((n_ + 31) / 32 + 1) * 4);
    return per_q * nq + pool + bitmaps + rerun;
  }

  void dispatch_loop() {
    cudaSetDevice(im_.device);
    for (;;) {
      BatchSlot* slot = nullptr;
      std::vector<ServerRequest*> take;
      {
        std::unique_lock<std::mutex> lk(mu_);
        for (;;) {
          if (stop_ && pending_.empty()) return;
          if (!pending_.empty()) {
            for (auto& s : slots_)
              if (!s.inflight) {
                slot = &s;
                break;
              }
            if (slot) {
              // admit FIFO requests up to the batch size, then check the budget
              uint64_t nq = 0;
              uint32_t kmax = 0, efmax = 0;
              size_t cnt = 0;
              while (cnt < pending_.size()) {
                ServerRequest* r = pending_[cnt];
                if (cnt > 0 && nq + r->nq > max_batch_) break;
                nq += r->nq;
                kmax = std::max(kmax, r->k);
                efmax = std::max(efmax, std::max(r->ef ? r->ef : ef_default_, r->k));
                ++cnt;
              }
              const uint64_t need = batch_bytes(nq, kmax, efmax);
              if (inflight_bytes_ + need <= budget_ || inflight_bytes_ == 0) {
                take.assign(pending_.begin(), pending_.begin() + static_cast<long>(cnt));
                pending_.erase(pending_.begin(), pending_.begin() + static_cast<long>(cnt));
                slot->bytes = need;
                inflight_bytes_ += need;
                slot->inflight = true;
                break;
              }
              ++memory_waits_;
              slot = nullptr;
            }
          }
          cv_.wait(lk);
        }
      }
      launch(*slot, take);
    }
  }

  void launch(BatchSlot& s, std::vector<ServerRequest*>& take) {
    uint64_t nq = 0;
    uint32_t kstride = 0;
    for (auto* r : take) {
      nq += r->nq;
      kstride = std::max(kstride, r->k);
    }
    s.reqs = take;
    s.kstride = kstride;
    s.offset.assign(take.size(), 0);
    s.efq.assign(nq, 0);
    s.kq.assign(nq, 0);
    s.fsel.assign(nq, -1);
    s.ftab.clear();
    bool ok = s.q.ensure(nq * dim_) && s.out.ensure(nq * kstride, true) && s.done.ensure(nq, true);
    if (ok) std::memset(s.done.p, 0, nq * sizeof(uint32_t));
    s.req_done.assign(take.size(), 0);
    s.ndone = 0;
    uint64_t row = 0;
    for (size_t i = 0; ok && i < take.size(); ++i) {
      ServerRequest* r = take[i];
      s.offset[i] = static_cast<uint32_t>(row);
      std::memcpy(s.q.p + row * dim_, r->queries, sizeof(float) * r->nq * dim_);
      int32_t f = -1;
      if (r->has_filter) {
        f = static_cast<int32_t>(s.ftab.size());
        s.ftab.push_back(r->filter.view);
      }
      for (uint32_t j = 0; j < r->nq; ++j) {
        s.efq[row + j] = r->ef;
        s.kq[row + j] = r->k;
        s.fsel[row + j] = f;
      }
      row += r->nq;
    }
    int rc = ok ? HGD_OK : HGD_ENOMEM;
    std::string err = ok ? "" : "server: cannot allocate pinned staging";
    if (ok) {
      hgd_search_args a{};
      a.queries = s.q.p;
      a.nq = nq;
      a.k = kstride;
      a.ef = 0;
      a.ef_default = ef_default_;
      a.precision = static_cast<uint32_t>(precision_);
      a.ef_per_query = s.efq.data();
      a.k_per_query = s.kq.data();
      a.filters = s.ftab.empty() ? nullptr : s.ftab.data();
      a.num_filters = static_cast<uint32_t>(s.ftab.size());
      a.filter_of_query = s.ftab.empty() ? nullptr : s.fsel.data();
      a.out = s.out.dev;
      a.out_on_device = 1;
      a.done_flags = s.done.dev;
      a.filter_scan_permille = filter_scan_permille_;
      a.rerank_factor = rerank_factor_;
      a.warps_per_query = warps_per_query_;
      a.lists_per_step = lists_per_step_;
      a.filter_scan_mode = filter_scan_mode_;
      a.stream = s.stream;
      a.synchronize = 0;
      rc = hgd_search(g_, &a);
      if (rc != HGD_OK) err = hgd_last_error();
      if (rc == HGD_OK && cudaEventRecord(s.ev, s.stream) != cudaSuccess) {
        rc = HGD_ECUDA;
        err = "server: cudaEventRecord failed";
      }
    }
    std::lock_guard<std::mutex> lk(mu_);
    ++batches_;
    batch_queries_ += nq;
    if (rc != HGD_OK) {  // fail the batch's requests, free the slot
      for (auto* r : take) {
        r->status = rc == HGD_EINVAL ? HG_EINVAL : HG_ERUNTIME;
        r->error = err;
        r->done = true;
      }
      inflight_bytes_ -= s.bytes;
      s.inflight = false;
      s.reqs.clear();
      cv_done_.notify_all();
      cv_.notify_all();
      return;
    }
    launched_.push_back(&s);
    cv_launched_.notify_one();
  }

  // Returns every request of a launched batch whose done flags are all up,
  // and frees the slot once all its requests are out and its work is over.
  void complete_loop() {
    cudaSetDevice(im_.device);
    std::vector<BatchSlot*> snapshot;
    std::vector<ServerRequest*> finished;
    for (;;) {
      {
        std::unique_lock<std::mutex> lk(mu_);
        // nothing in flight: sleep until a batch is launched (or the server stops)
        cv_launched_.wait(lk, [&] { return stop_ || !launched_.empty(); });
        if (stop_ && launched_.empty() && pending_.empty()) {
          bool any = false;
          for (auto& s : slots_) any = any || s.inflight;
          if (!any) return;
        }
        snapshot = launched_;
      }
      bool progress = false;
      for (BatchSlot* s : snapshot) {
        finished.clear();
        const bool gpu_done = s->ndone == s->reqs.size() || cudaEventQuery(s->ev) != cudaErrorNotReady;
        for (size_t i = 0; i < s->reqs.size(); ++i) {
          if (s->req_done[i]) continue;
          ServerRequest* r = s->reqs[i];
          const uint32_t* f = s->done.p + s->offset[i];
          bool all = true;
          for (uint32_t j = 0; j < r->nq && all; ++j) all = __atomic_load_n(f + j, __ATOMIC_ACQUIRE) != 0u;
          if (!all) {
            if (!gpu_done) continue;
            // the batch is over but this request's rows never arrived
            r->status = HG_ERUNTIME;
            r->error = "server: batch ended without finishing a request";
          } else {
            for (uint32_t j = 0; j < r->nq; ++j)
              std::memcpy(r->out + static_cast<size_t>(j) * r->k,
                          s->out.p + static_cast<size_t>(s->offset[i] + j) * s->kstride, sizeof(hg_neighbor) * r->k);
          }
          s->req_done[i] = 1;
          ++s->ndone;
          finished.push_back(r);
        }
        const bool slot_free = s->ndone == s->reqs.size() && cudaEventQuery(s->ev) != cudaErrorNotReady;
        if (finished.empty() && !slot_free) continue;
        progress = true;
        const auto now = Clock::now();
        std::lock_guard<std::mutex> lk(mu_);
        for (ServerRequest* r : finished) {
          r->latency_ms = std::chrono::duration<double, std::milli>(now - r->arrival).count();
          r->done = true;
          if (r->status == HG_OK) {
            lat_.push_back(r->latency_ms);
            queries_done_ += r->nq;
            if (!have_first_ || r->arrival < first_arrival_) first_arrival_ = r->arrival;
            have_first_ = true;
            last_done_ = now;
          }
        }
        if (slot_free) {
          launched_.erase(std::find(launched_.begin(), launched_.end(), s));
          inflight_bytes_ -= s->bytes;
          s->inflight = false;
          s->reqs.clear();
          cv_.notify_all();
        }
        cv_done_.notify_all();
      }
      // batches in flight: poll their done flags without sleeping (a sleep's
      // timer slack, tens of microseconds, would add to every request)
      if (!progress) std::this_thread::yield();
    }
  }

  const Index::Impl& im_;
  hgd_graph* g_ = nullptr;
  uint32_t dim_ = 0, ef_default_ = 10, max_inflight_ = 4, max_batch_ = 4096;
  size_t n_ = 0;
  int precision_ = 0;
  uint32_t filter_scan_permille_ = 0;
  uint32_t rerank_factor_ = 0;
  uint32_t warps_per_query_ = 1;
  uint32_t lists_per_step_ = 0;
  uint32_t filter_scan_mode_ = 0;
  uint64_t budget_ = 0, inflight_bytes_ = 0;
  std::mutex mu_;
  std::condition_variable cv_, cv_done_, cv_launched_;
  std::deque<ServerRequest*> pending_;
  std::unordered_map<uint64_t, std::unique_ptr<ServerRequest>> reqs_;
  std::vector<BatchSlot> slots_;
  std::vector<BatchSlot*> launched_;
  uint64_t next_ticket_ = 0;
  bool stop_ = false;
  std::thread dispatcher_, completer_;
  // stats
  std::vector<double> lat_;
  uint64_t queries_done_ = 0, batches_ = 0, batch_queries_ = 0, memory_waits_ = 0;
  Clock::time_point first_arrival_, last_done_;
  bool have_first_ = false;

 public:
  // Submit each request at its arrival time (seconds from the call), wait for
  // all, and report the stats of exactly these requests.
  void replay(const hg_request* reqs, const double* arrival_s, size_t n, hg_server_stats* out, double* latency_ms) {
    reset_stats();
    std::vector<uint64_t> tickets(n);
    const auto t0 = Clock::now();
    for (size_t i = 0; i < n; ++i) {
      const auto when = t0 + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(arrival_s[i]));
      auto now = Clock::now();
      if (when > now + std::chrono::microseconds(200)) std::this_thread::sleep_until(when - std::chrono::microseconds(100));
      while (Clock::now() < when) {
      }
      tickets[i] = submit(reqs[i], when);
    }
    for (size_t i = 0; i < n; ++i) {
      int st = HG_OK;
      std::string err;
      wait(tickets[i], latency_ms ? latency_ms + i : nullptr, &st, &err);
      if (st != HG_OK) throw std::runtime_error("server replay: request failed: " + err);
    }
    stats(out);
  }
};

}  // namespace hnsw::gb

namespace hnsw::gb {

Server* server_new(const Index::Impl& im, const hg_server_config& cfg) {
  if (im.count == 0) throw std::invalid_argument("server: empty index");
  return new Server(im, cfg);
}
void server_delete(Server* s) { delete s; }
uint64_t server_submit(Server* s, const hg_request& r) { return s->submit(r, Clock::now()); }
void server_wait(Server* s, uint64_t ticket, double* latency_ms) {
  int st = HG_OK;
  std::string err;
  s->wait(ticket, latency_ms, &st, &err);
  if (st == HG_EINVAL) throw std::invalid_argument(err);
  if (st != HG_OK) throw std::runtime_error(err);
}
void server_replay(Server* s, const hg_request* reqs, const double* arrival_s, size_t n, hg_server_stats* out,
                   double* latency_ms) {
  s->replay(reqs, arrival_s, n, out, latency_ms);
}
void server_stats(Server* s, hg_server_stats* out) { s->stats(out); }

}  // namespace hnsw::gb
