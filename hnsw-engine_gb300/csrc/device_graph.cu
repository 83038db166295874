// device_graph.cu -- the hgd_* C ABI: graph mirror in HBM and batch launches.
//
// HBM layout of a graph (all arrays resident for the index's lifetime):
//   vecs    n x pd float32, 64-byte rows (pd = dim rounded up to 16)
//   l0      n x l0s uint32 ids, l0s = 2M rounded up to 16 (M = 16: 128 B, one
//           aligned line per list); unused slots hold 0xFFFFFFFF, so the
//           count word of the file layout is not needed
//   up      per node with level L >= 1, L blocks of ups = M rounded up to 16
//           ids (M = 16: 64 B), padded the same way; up_blk[id] = first block
//   labels  n x uint64 (read only when writing results)
//   alive   n bits, 1 = not deleted (soft deletes flip one bit)
// Per call: queries, per-query ef / k, filter bitsets translated to internal
// ids, the work-queue counter and per-warp scratch (spill pool, visited bitmap).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "bf_mma.h"
#include "hnswgpu_device.h"
#include "search_common.cuh"

namespace hg {
int slots_for(uint32_t pd);
cudaError_t launch_inv_norm(const float* qs, uint32_t nq, uint32_t dim, float* out, cudaStream_t st);
cudaError_t launch_search(const SearchParams& P, const float* inv, int blocks, int warps_per_block, cudaStream_t st);
int search_occupancy(uint32_t pd, int metric, int order, int warps_per_block, uint32_t H, uint32_t R, uint32_t C);
cudaError_t launch_search_approx(const SearchParams& P, const float* inv, int blocks, int wpb, cudaStream_t st);
int occupancy_approx(uint32_t pdc, int metric, int prec, int order, int wpb, size_t smem);
cudaError_t launch_search_wide(const SearchParams& P, const float* inv, int blocks, cudaStream_t st);
int occupancy_wide(int metric, int prec, int order, uint32_t R);
cudaError_t launch_encode(const float* vecs, uint32_t n, uint32_t pd, uint32_t pdc, int prec, void* out,
                          float* scale, float* aux, cudaStream_t st);
cudaError_t launch_search_beam(const SearchParams& P, const float* inv, int blocks, int wpb, bool filt,
                               cudaStream_t st);
int occupancy_beam(int metric, int prec, int order, int wpb, size_t smem, bool filt);
cudaError_t launch_bucket(const uint32_t* efq, const uint32_t* kq, uint32_t nq, uint32_t ef_all, uint32_t ef_default,
                          uint32_t k_all, const BucketSpec& spec, uint32_t* counts, uint32_t* lists, cudaStream_t st,
                          const uint8_t* skip);
cudaError_t launch_translate_filter(const uint64_t* label_words, uint64_t num_bits, const uint64_t* labels, uint32_t n,
                                    uint32_t* out, cudaStream_t st);
int build_graph(hgd_build_args* a, int device, std::string* err);
cudaError_t launch_relayout_l0(const uint32_t* raw, uint64_t n, uint32_t M0, uint32_t* l0, uint32_t l0s, uint32_t* dup,
                               cudaStream_t st);
}  // namespace hg

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

#define HG_CUDA(call)                                                                              \
  do {                                                                                             \
    cudaError_t e_ = (call);                                                                       \
    if (e_ != cudaSuccess) {                                                                       \
      return fail(e_ == cudaErrorMemoryAllocation ? HGD_ENOMEM : HGD_ECUDA,                        \
                  std::string(#call) + ": " + cudaGetErrorString(e_));                             \
    }                                                                                              \
  } while (0)

// A grow-only device buffer.
struct DBuf {
  void* p = nullptr;
  size_t bytes = 0;
  cudaError_t ensure(size_t need) {
    if (need <= bytes) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    size_t n = std::max<size_t>(need, 256);
    cudaError_t e = cudaMalloc(&p, n);
    if (e == cudaSuccess) bytes = n;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  template <typename T>
  T* as() const {
    return static_cast<T*>(p);
  }
};

struct PinnedBuf {
  void* p = nullptr;
  size_t bytes = 0;
  cudaError_t ensure(size_t need) {
    if (need <= bytes) return cudaSuccess;
    if (p) cudaFreeHost(p);
    p = nullptr;
    bytes = 0;
    size_t n = std::max<size_t>(need, 256);
    cudaError_t e = cudaMallocHost(&p, n);
    if (e == cudaSuccess) bytes = n;
    return e;
  }
  void release() {
    if (p) cudaFreeHost(p);
    p = nullptr;
    bytes = 0;
  }
};

uint32_t round_up(uint32_t v, uint32_t m) { return (v + m - 1) / m * m; }
uint32_t next_pow2(uint32_t v) {
  uint32_t p = 1;
  while (p < v) p <<= 1;
  return p;
}

}  // namespace

namespace hg {
void set_last_error(const std::string& msg) { g_err = msg; }
}  // namespace hg

// Scratch of one batch in flight.  A batch takes a free workspace and makes
// its stream wait for the workspace's previous batch (event `done`), so
// batches on different streams overlap on the GPU without sharing buffers.
struct Workspace {
  DBuf q, efq, kq, fsel, fptrs, fbits, inv, out, nres, counters;
  DBuf work;  // [1] overflow count [2] rerun work [4] error [8+b] bucket work [32+b] bucket size
  DBuf ovf_list, pool, pool_t2, bitmaps, pool_big, bitmaps_big, owners, lists, pool_ids, pool_n;
  PinnedBuf pin_in, pin_out;
  std::vector<cudaStream_t> aux;  // one per ef bucket
  std::vector<cudaEvent_t> ev_join;
  cudaEvent_t ev_fork = nullptr;
  cudaEvent_t done = nullptr;  // recorded after the batch's last use of this workspace
  bool busy = false;
  // CUDA graph of one device-resident batch shape: captured on the second call
  // with the same key, replayed after that
  std::string graph_seen, graph_key;
  cudaGraphExec_t graph_exec = nullptr;
  // queries routed to the exact scan: list, filter per entry, skip flags; the
  // scan's scratch and stream
  DBuf scan_qlist, scan_fsel, scan_route;
  hg::bfm::Scratch* scan_sc = nullptr;
  cudaStream_t scan_stream = nullptr;
  cudaEvent_t scan_fork = nullptr, scan_join = nullptr;
  void release_all() {
    for (DBuf* d : {&q, &efq, &kq, &fsel, &fptrs, &fbits, &inv, &out, &nres, &counters, &work, &ovf_list, &pool, &pool_t2,
                    &bitmaps, &pool_big, &bitmaps_big, &owners, &lists, &pool_ids, &pool_n})
      d->release();
    pin_in.release();
    pin_out.release();
    for (cudaStream_t s2 : aux) cudaStreamDestroy(s2);
    for (cudaEvent_t e2 : ev_join) cudaEventDestroy(e2);
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (done) cudaEventDestroy(done);
    if (graph_exec) cudaGraphExecDestroy(graph_exec);
    graph_exec = nullptr;
    graph_key.clear();
    graph_seen.clear();
    scan_qlist.release();
    scan_fsel.release();
    scan_route.release();
    hg::bfm::scratch_free(scan_sc);
    scan_sc = nullptr;
    if (scan_stream) cudaStreamDestroy(scan_stream);
    if (scan_fork) cudaEventDestroy(scan_fork);
    if (scan_join) cudaEventDestroy(scan_join);
    scan_stream = nullptr;
    scan_fork = scan_join = nullptr;
    aux.clear();
    ev_join.clear();
    ev_fork = done = nullptr;
  }
  uint64_t bytes() const {
    uint64_t t = 0;
    for (const DBuf* d : {&q, &efq, &kq, &fsel, &fptrs, &fbits, &inv, &out, &nres, &counters, &work, &ovf_list,
                          &pool, &pool_t2, &bitmaps, &pool_big, &bitmaps_big, &owners, &lists, &pool_ids, &pool_n})
      t += d->bytes;
    return t;
  }
};

struct hgd_graph {
  int device = 0;
  int order = HGD_ORDER_AVX512;
  int sms = 0;
  cudaStream_t stream = nullptr;
  std::mutex mu;  // one batch at a time per graph (its scratch is shared)
  // graph
  uint64_t n = 0, dim = 0, pd = 0, M = 0;
  int metric = 0, max_level = -1;
  uint32_t entry = hg::kNoId;
  uint32_t l0s = 0, ups = 0;
  bool identity_labels = true, dedup = false;
  uint64_t num_deleted = 0;
  DBuf vecs, l0, up, up_blk, labels, alive;
  std::vector<uint32_t> alive_host;
  // compressed copies for FP16 / FP8 traversal (built on first use)
  DBuf v16, v8, vscale, vaux16, vaux8;
  bool has16 = false, has8 = false;
  // batch scratch
  std::mutex ws_mu;
  std::vector<std::unique_ptr<Workspace>> ws;
  PinnedBuf pin_patch;  // tombstone word staging
  // FP16 copy of the rows for the exact scan of routed filtered queries (built on first use)
  hg::bfm::Store* scan = nullptr;
  // autotuned launch shapes (guarded by ws_mu); version enters graph keys
  std::vector<hgd_tune_entry> tune;
  int launch_mode = HGD_LAUNCH_BUCKETS;
  uint64_t tune_version = 0;
};

namespace {

// Takes a workspace that no host thread is using (creating one if needed) and
// gives it back when the call returns; GPU-side reuse is ordered by `done`.
class WorkspaceLease {
 public:
  // Prefers a workspace whose previous batch has finished; otherwise opens a
  // new one (up to kMaxWorkspaces batches in flight), else waits for the
  // oldest.  Buffers may then be grown safely: nothing on the GPU uses them.
  static constexpr size_t kMaxWorkspaces = 16;
  explicit WorkspaceLease(hgd_graph* g, const std::string* graph_key = nullptr) : g_(g) {
    Workspace* wait_for = nullptr;
    {
      std::lock_guard<std::mutex> lk(g->ws_mu);
      if (graph_key)  // a workspace holding this batch's graph (or about to capture it) comes first
        for (auto& w : g->ws)
          if (!w->busy && (w->graph_key == *graph_key || w->graph_seen == *graph_key) &&
              cudaEventQuery(w->done) == cudaSuccess) {
            w_ = w.get();
            break;
          }
      if (!w_)
        for (auto& w : g->ws)
          if (!w->busy && cudaEventQuery(w->done) == cudaSuccess) {
            w_ = w.get();
            break;
          }
      if (!w_ && g->ws.size() < kMaxWorkspaces) {
        auto nw = std::make_unique<Workspace>();
        if (cudaEventCreateWithFlags(&nw->done, cudaEventDisableTiming) != cudaSuccess) return;
        w_ = nw.get();
        g->ws.push_back(std::move(nw));
      }
      if (!w_)
        for (auto& w : g->ws)
          if (!w->busy) {
            w_ = wait_for = w.get();
            break;
          }
      if (w_) w_->busy = true;
    }
    if (wait_for) cudaEventSynchronize(wait_for->done);
  }
  ~WorkspaceLease() {
    if (!w_) return;
    if (st_set_) cudaEventRecord(w_->done, st_);  // after everything this call enqueued
    std::lock_guard<std::mutex> lk(g_->ws_mu);
    w_->busy = false;
  }
  Workspace* get() const { return w_; }
  void on_stream(cudaStream_t st) {
    st_ = st;
    st_set_ = true;
  }

 private:
  hgd_graph* g_;
  Workspace* w_ = nullptr;
  cudaStream_t st_ = nullptr;
  bool st_set_ = false;
};

// The inputs a captured batch depends on: pointers, sizes, shape fields, the
// tombstone switch and the tuning table in force.
std::string graph_key_of(const hgd_search_args* a, bool any_deleted, uint64_t tune_version) {
  char buf[512];
  std::snprintf(buf, sizeof buf, "%p/%llu/%u/%u/%u/%u/%p/%p/%p/%p/%p/%u/%u/%u/%u/%d/%llu",
                static_cast<const void*>(a->queries), static_cast<unsigned long long>(a->nq), a->k, a->ef,
                a->ef_default, a->precision, static_cast<const void*>(a->ef_per_query),
                static_cast<const void*>(a->k_per_query), a->out, static_cast<const void*>(a->nres),
                static_cast<const void*>(a->done_flags), a->hash_slots, a->cand_cap, a->warps_per_block, a->pool_cap,
                any_deleted ? 1 : 0, static_cast<unsigned long long>(tune_version));
  return buf;
}

int enqueue_batch(hgd_graph* g, const hgd_search_args* a, Workspace* w, cudaStream_t st);

int check_view(const hgd_graph_view* v, int order, const char* who) {
  const std::string w(who);
  if (order != HGD_ORDER_AVX512 && order != HGD_ORDER_NEON)
    return fail(HGD_EINVAL, w + ": the GPU implements the AVX-512 and NEON summation orders only");
  if (v->count >= 0xFFFFFFFFull) return fail(HGD_EINVAL, w + ": count exceeds 32-bit ids");
  if (v->padded_dim % 16 != 0 || v->padded_dim < v->dim || v->dim == 0)
    return fail(HGD_EINVAL, w + ": padded_dim must be dim rounded up to 16");
  if (hg::slots_for(static_cast<uint32_t>(v->padded_dim)) > 33)
    return fail(HGD_EINVAL, w + ": padded dimension above 1024 is not supported on the GPU");
  if (v->M < 2 || v->M > 2048) return fail(HGD_EINVAL, w + ": invalid M");
  return HGD_OK;
}

// A graph with its sizes, device and stream set, no arrays yet.
int graph_begin(const hgd_graph_view* v, int device, int order, hgd_graph** out) {
  auto* g = new hgd_graph();
  g->device = device;
  g->order = order;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&g->sms, cudaDevAttrMultiProcessorCount, device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    hgd_graph_free(g);
    return fail(HGD_ECUDA, std::string("graph setup: ") + cudaGetErrorString(e));
  }
  g->n = v->count;
  g->dim = v->dim;
  g->pd = v->padded_dim;
  g->M = v->M;
  g->metric = v->metric;
  g->max_level = v->max_level;
  g->entry = v->entry_point;
  g->l0s = round_up(static_cast<uint32_t>(2 * v->M), 16);
  g->ups = round_up(static_cast<uint32_t>(v->M), 16);
  *out = g;
  return HGD_OK;
}

int up_copy(DBuf& d, const void* src, size_t bytes) {
  cudaError_t e = d.ensure(std::max<size_t>(bytes, 16));
  if (e != cudaSuccess) return fail(HGD_ENOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  if (bytes) {
    e = cudaMemcpy(d.p, src, bytes, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return fail(HGD_ECUDA, std::string("cudaMemcpy: ") + cudaGetErrorString(e));
  }
  return HGD_OK;
}

// The small parts, built on the host from the view and uploaded: the upper
// layers in blocks of ups ids per (node, level) with each node's first
// block, the alive bits, whether labels are the ids, and whether a list
// holds an id twice (layer 0 too when check_l0).
int graph_small_parts(hgd_graph* g, const hgd_graph_view* v, bool check_l0) {
  const uint64_t n = v->count;
  const uint32_t M0 = static_cast<uint32_t>(2 * v->M);
  std::vector<uint32_t> mark(n, hg::kNoId);
  uint64_t list_no = 0;
  auto dup_check = [&](const uint32_t* ids, uint32_t cnt) {
    for (uint32_t j = 0; j < cnt; ++j) {
      if (mark[ids[j]] == static_cast<uint32_t>(list_no)) g->dedup = true;
      mark[ids[j]] = static_cast<uint32_t>(list_no);
    }
    ++list_no;
  };
  if (check_l0)
    for (uint64_t i = 0; i < n; ++i) {
      const uint32_t* src = v->level0 + i * (1 + M0);
      dup_check(src + 1, std::min(src[0], M0));
    }
  std::vector<uint32_t> up_blk(n, hg::kNoId);
  uint64_t blocks = 0;
  for (uint64_t i = 0; i < n; ++i) blocks += v->levels[i];
  std::vector<uint32_t> up(std::max<uint64_t>(blocks, 1) * g->ups, hg::kNoId);
  uint64_t b = 0;
  for (uint64_t i = 0; i < n; ++i) {
    const int L = v->levels[i];
    if (L == 0) continue;
    up_blk[i] = static_cast<uint32_t>(b);
    for (int lc = 1; lc <= L; ++lc, ++b) {
      const uint32_t* src = v->upper + v->upper_offset[i] + static_cast<uint64_t>(lc - 1) * (1 + v->M);
      const uint32_t cnt = std::min<uint32_t>(src[0], static_cast<uint32_t>(v->M));
      std::memcpy(&up[b * g->ups], src + 1, cnt * 4);
      dup_check(src + 1, cnt);
    }
  }
  g->identity_labels = true;
  for (uint64_t i = 0; i < n && g->identity_labels; ++i) g->identity_labels = v->labels[i] == i;
  g->alive_host.assign((n + 31) / 32 + 1, 0u);
  g->num_deleted = 0;
  for (uint64_t i = 0; i < n; ++i) {
    if (v->deleted[i] == 0) g->alive_host[i >> 5] |= 1u << (i & 31);
    else ++g->num_deleted;
  }
  int rc;
  if ((rc = up_copy(g->up, up.data(), up.size() * 4)) != HGD_OK) return rc;
  if ((rc = up_copy(g->up_blk, up_blk.data(), up_blk.size() * 4)) != HGD_OK) return rc;
  return up_copy(g->alive, g->alive_host.data(), g->alive_host.size() * 4);
}

}  // namespace

// Streamed upload state: the graph under construction, a ring of pinned
// staging buffers with the event of each one's last copy, and layer 0 in the
// file's layout until it is re-laid on the device.
constexpr int kStreamBuffers = 4;
struct hgd_stream {
  hgd_graph* g = nullptr;
  uint32_t M0 = 0;
  uint64_t chunk = 0;
  uint64_t sec_bytes[3] = {0, 0, 0};
  uint64_t submitted[3] = {0, 0, 0};
  std::vector<PinnedBuf> ring;
  std::vector<cudaEvent_t> ev;
  int cur = kStreamBuffers - 1;
  bool handed = false;
  DBuf raw_l0, flag;
};

extern "C" {

const char* hgd_last_error(void) { return g_err.c_str(); }

int hgd_build_graph(hgd_build_args* args, int device) {
  std::string err;
  const int rc = hg::build_graph(args, device, &err);
  return rc == HGD_OK ? rc : fail(rc, err);
}

int hgd_graph_upload(const hgd_graph_view* v, int device, int order, hgd_graph** out) {
  if (!v || !out) return fail(HGD_EINVAL, "hgd_graph_upload: null argument");
  int rc = check_view(v, order, "hgd_graph_upload");
  if (rc != HGD_OK) return rc;
  hgd_graph* g = nullptr;
  if ((rc = graph_begin(v, device, order, &g)) != HGD_OK) return rc;
  auto cleanup = [&](int code) {
    hgd_graph_free(g);
    return code;
  };
  const uint64_t n = v->count;
  const uint32_t M0 = static_cast<uint32_t>(2 * v->M);
  // host re-layout of layer 0
  std::vector<uint32_t> l0(static_cast<size_t>(n) * g->l0s, hg::kNoId);
  for (uint64_t i = 0; i < n; ++i) {
    const uint32_t* src = v->level0 + i * (1 + M0);
    const uint32_t cnt = std::min(src[0], M0);
    std::memcpy(&l0[i * g->l0s], src + 1, cnt * 4);
  }
  if ((rc = graph_small_parts(g, v, true)) != HGD_OK) return cleanup(rc);
  if ((rc = up_copy(g->vecs, v->vectors, n * g->pd * 4)) != HGD_OK) return cleanup(rc);
  if ((rc = up_copy(g->l0, l0.data(), l0.size() * 4)) != HGD_OK) return cleanup(rc);
  if ((rc = up_copy(g->labels, v->labels, n * 8)) != HGD_OK) return cleanup(rc);
  *out = g;
  return HGD_OK;
}

// ---- streamed upload -------------------------------------------------------
int hgd_stream_begin(const hgd_graph_view* v, int device, int order, uint64_t chunk_bytes, hgd_stream** out) {
  if (!v || !out) return fail(HGD_EINVAL, "hgd_stream_begin: null argument");
  int rc = check_view(v, order, "hgd_stream_begin");
  if (rc != HGD_OK) return rc;
  if (v->count > 0xFFFFFFFFull - 64) return fail(HGD_EINVAL, "hgd_stream_begin: count exceeds 32-bit ids");
  if (chunk_bytes < 4096 || chunk_bytes % 16 != 0)
    return fail(HGD_EINVAL, "hgd_stream_begin: chunk_bytes must be a multiple of 16, at least 4096");
  auto* s = new hgd_stream();
  if ((rc = graph_begin(v, device, order, &s->g)) != HGD_OK) {
    delete s;
    return rc;
  }
  auto cleanup = [&](int code) {
    hgd_stream_abort(s);
    return code;
  };
  const uint64_t n = v->count;
  s->M0 = static_cast<uint32_t>(2 * v->M);
  s->sec_bytes[0] = n * s->g->pd * 4;
  s->sec_bytes[1] = n * (1 + static_cast<uint64_t>(s->M0)) * 4;
  s->sec_bytes[2] = n * 8;
  DBuf* dst[3] = {&s->g->vecs, &s->raw_l0, &s->g->labels};
  for (int i = 0; i < 3; ++i) {
    const cudaError_t e = dst[i]->ensure(std::max<uint64_t>(s->sec_bytes[i], 16));
    if (e != cudaSuccess) return cleanup(fail(HGD_ENOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e)));
  }
  s->ring.resize(kStreamBuffers);
  s->ev.assign(kStreamBuffers, nullptr);
  for (int i = 0; i < kStreamBuffers; ++i) {
    cudaError_t e = s->ring[i].ensure(chunk_bytes);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->ev[i], cudaEventDisableTiming);
    if (e != cudaSuccess) return cleanup(fail(HGD_ENOMEM, std::string("pinned staging: ") + cudaGetErrorString(e)));
  }
  s->chunk = chunk_bytes;
  *out = s;
  return HGD_OK;
}

int hgd_stream_buffer(hgd_stream* s, void** buf, uint64_t* cap) {
  if (!s || !buf || !cap) return fail(HGD_EINVAL, "hgd_stream_buffer: null argument");
  const int next = (s->cur + 1) % kStreamBuffers;
  const cudaError_t e = cudaEventSynchronize(s->ev[next]);  // its previous copy (none yet: returns at once)
  if (e != cudaSuccess) return fail(HGD_ECUDA, std::string("hgd_stream_buffer: ") + cudaGetErrorString(e));
  s->cur = next;
  s->handed = true;
  *buf = s->ring[next].p;
  *cap = s->chunk;
  return HGD_OK;
}

int hgd_stream_submit(hgd_stream* s, int section, uint64_t offset, uint64_t bytes) {
  if (!s) return fail(HGD_EINVAL, "hgd_stream_submit: null stream");
  if (!s->handed) return fail(HGD_EINVAL, "hgd_stream_submit: no buffer taken");
  if (section < 0 || section > 2) return fail(HGD_EINVAL, "hgd_stream_submit: section must be 0, 1 or 2");
  if (bytes > s->chunk || offset > s->sec_bytes[section] || bytes > s->sec_bytes[section] - offset)
    return fail(HGD_EINVAL, "hgd_stream_submit: chunk outside the section");
  s->handed = false;
  if (bytes == 0) return HGD_OK;
  void* dst = section == 0 ? s->g->vecs.p : (section == 1 ? s->raw_l0.p : s->g->labels.p);
  cudaError_t e = cudaMemcpyAsync(static_cast<char*>(dst) + offset, s->ring[s->cur].p, bytes, cudaMemcpyHostToDevice,
                                  s->g->stream);
  if (e == cudaSuccess) e = cudaEventRecord(s->ev[s->cur], s->g->stream);
  if (e != cudaSuccess) return fail(HGD_ECUDA, std::string("hgd_stream_submit: ") + cudaGetErrorString(e));
  s->submitted[section] += bytes;
  return HGD_OK;
}

int hgd_stream_finish(hgd_stream* s, const hgd_graph_view* v, hgd_graph** out) {
  if (!s || !v || !out) return fail(HGD_EINVAL, "hgd_stream_finish: null argument");
  auto cleanup = [&](int code) {
    hgd_stream_abort(s);
    return code;
  };
  hgd_graph* g = s->g;
  if (v->count != g->n || v->padded_dim != g->pd || v->M != g->M)
    return cleanup(fail(HGD_EINVAL, "hgd_stream_finish: the view does not match hgd_stream_begin's"));
  for (int i = 0; i < 3; ++i)
    if (s->submitted[i] != s->sec_bytes[i])
      return cleanup(fail(HGD_EINVAL, "hgd_stream_finish: a section was not streamed in full"));
  const uint64_t n = g->n;
  cudaError_t e = g->l0.ensure(std::max<uint64_t>(n * g->l0s * 4, 16));
  if (e != cudaSuccess) return cleanup(fail(HGD_ENOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e)));
  // layer 0 into the padded stride on the device; duplicate ids in a list
  // (M0 <= 32: one warp compare per list) raise the flag
  const bool dev_dups = s->M0 <= 32;
  int rc = graph_small_parts(g, v, !dev_dups);
  if (rc != HGD_OK) return cleanup(rc);
  if ((e = s->flag.ensure(16)) != cudaSuccess) return cleanup(fail(HGD_ENOMEM, cudaGetErrorString(e)));
  if ((e = cudaMemsetAsync(s->flag.p, 0, 16, g->stream)) != cudaSuccess)
    return cleanup(fail(HGD_ECUDA, cudaGetErrorString(e)));
  if (n > 0) {
    if ((e = hg::launch_relayout_l0(s->raw_l0.as<uint32_t>(), n, s->M0, g->l0.as<uint32_t>(), g->l0s,
                                    dev_dups ? s->flag.as<uint32_t>() : nullptr, g->stream)) != cudaSuccess)
      return cleanup(fail(HGD_ECUDA, std::string("layer-0 re-layout: ") + cudaGetErrorString(e)));
  }
  uint32_t dup = 0;
  if ((e = cudaMemcpyAsync(&dup, s->flag.p, 4, cudaMemcpyDeviceToHost, g->stream)) != cudaSuccess ||
      (e = cudaStreamSynchronize(g->stream)) != cudaSuccess)
    return cleanup(fail(HGD_ECUDA, std::string("hgd_stream_finish: ") + cudaGetErrorString(e)));
  if (dup) g->dedup = true;
  s->g = nullptr;
  hgd_stream_abort(s);  // frees the staging, not the graph
  *out = g;
  return HGD_OK;
}

void hgd_stream_abort(hgd_stream* s) {
  if (!s) return;
  if (s->g) {
    hgd_graph_free(s->g);  // synchronises the stream first
  } else {
    for (cudaEvent_t e : s->ev)
      if (e) cudaEventSynchronize(e);
  }
  for (cudaEvent_t e : s->ev)
    if (e) cudaEventDestroy(e);
  for (auto& b : s->ring) b.release();
  s->raw_l0.release();
  s->flag.release();
  delete s;
}

int hgd_graph_set_order(hgd_graph* g, int order) {
  if (!g) return fail(HGD_EINVAL, "hgd_graph_set_order: null graph");
  if (order != HGD_ORDER_AVX512 && order != HGD_ORDER_NEON)
    return fail(HGD_EINVAL, "hgd_graph_set_order: the GPU implements the AVX-512 and NEON summation orders only");
  g->order = order;
  return HGD_OK;
}

int hgd_graph_set_deleted(hgd_graph* g, uint32_t id, int deleted) {
  if (!g) return fail(HGD_EINVAL, "hgd_graph_set_deleted: null graph");
  if (id >= g->n) return fail(HGD_EINVAL, "hgd_graph_set_deleted: id out of range");
  std::lock_guard<std::mutex> lock(g->mu);
  uint32_t& word = g->alive_host[id >> 5];
  const uint32_t bit = 1u << (id & 31);
  const bool was_alive = (word & bit) != 0;
  if (deleted && was_alive) {
    word &= ~bit;
    ++g->num_deleted;
  } else if (!deleted && !was_alive) {
    word |= bit;
    --g->num_deleted;
  } else {
    return HGD_OK;
  }
  HG_CUDA(cudaSetDevice(g->device));
  HG_CUDA(g->pin_patch.ensure(8));
  std::memcpy(g->pin_patch.p, &word, 4);
  HG_CUDA(cudaMemcpyAsync(g->alive.as<uint32_t>() + (id >> 5), g->pin_patch.p, 4, cudaMemcpyHostToDevice, g->stream));
  HG_CUDA(cudaStreamSynchronize(g->stream));
  return HGD_OK;
}

void hgd_graph_free(hgd_graph* g) {
  if (!g) return;
  cudaSetDevice(g->device);
  if (g->stream) cudaStreamSynchronize(g->stream);
  for (auto& w : g->ws) {
    if (w->done) cudaEventSynchronize(w->done);
    w->release_all();
  }
  g->ws.clear();
  hg::bfm::store_free(g->scan);
  for (DBuf* d : {&g->vecs, &g->l0, &g->up, &g->up_blk, &g->labels, &g->alive, &g->v16, &g->v8, &g->vscale,
                  &g->vaux16, &g->vaux8})
    d->release();
  g->pin_patch.release();
  if (g->stream) cudaStreamDestroy(g->stream);
  delete g;
}

uint64_t hgd_graph_device_bytes(const hgd_graph* g) {
  if (!g) return 0;
  uint64_t t = 0;
  for (const DBuf* d : {&g->vecs, &g->l0, &g->up, &g->up_blk, &g->labels, &g->alive, &g->v16, &g->v8, &g->vscale,
                  &g->vaux16, &g->vaux8})
    t += d->bytes;
  for (const auto& w : g->ws) t += w->bytes();
  return t;
}

int hgd_search(hgd_graph* g, const hgd_search_args* a) {
  if (!g || !a) return fail(HGD_EINVAL, "hgd_search: null argument");
  if (a->k == 0) return fail(HGD_EINVAL, "search_batch: k must be > 0");
  if (a->nq == 0) return HGD_OK;
  if (!a->queries || !a->out) return fail(HGD_EINVAL, "search_batch: null pointer");
  if (a->nq >= 0xFFFFFFFFull) return fail(HGD_EINVAL, "hgd_search: too many queries in one batch");
  if (a->precision > HGD_PREC_FP8) return fail(HGD_EINVAL, "hgd_search: unknown precision");
  if (a->num_filters && !a->filters) return fail(HGD_EINVAL, "hgd_search: null filter table");
  HG_CUDA(cudaSetDevice(g->device));
  cudaStream_t st = a->stream ? static_cast<cudaStream_t>(a->stream) : g->stream;
  const bool graphable = a->use_graph && a->queries_on_device && a->out_on_device && !a->counters &&
                         a->num_filters == 0 && !a->synchronize;
  std::string key;
  if (graphable) {
    std::lock_guard<std::mutex> lk(g->ws_mu);
    key = graph_key_of(a, g->num_deleted > 0, g->tune_version);
  }
  WorkspaceLease lease(g, graphable ? &key : nullptr);
  Workspace* w = lease.get();
  if (!w) return fail(HGD_ERUNTIME, "hgd_search: no workspace available (all held by calls in progress)");
  HG_CUDA(cudaStreamWaitEvent(st, w->done, 0));  // its previous batch has finished with it
  lease.on_stream(st);
  if (!graphable) return enqueue_batch(g, a, w, st);
  if (w->graph_exec && w->graph_key == key) {
    HG_CUDA(cudaGraphLaunch(w->graph_exec, st));
    return HGD_OK;
  }
  if (w->graph_seen != key) {  // first call of this shape: run it (sizes every buffer)
    w->graph_seen = key;
    return enqueue_batch(g, a, w, st);
  }
  // second call: capture the batch, then launch the graph
  if (w->graph_exec) {
    HG_CUDA(cudaGraphExecDestroy(w->graph_exec));
    w->graph_exec = nullptr;
    w->graph_key.clear();
  }
  HG_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  const int rc = enqueue_batch(g, a, w, st);
  cudaGraph_t graph = nullptr;
  const cudaError_t ec = cudaStreamEndCapture(st, &graph);
  if (rc != HGD_OK) {
    if (graph) cudaGraphDestroy(graph);
    return rc;
  }
  if (ec != cudaSuccess) return fail(HGD_ECUDA, std::string("hgd_search: graph capture: ") + cudaGetErrorString(ec));
  cudaGraphExec_t exec = nullptr;
  const cudaError_t ei = cudaGraphInstantiateWithFlags(&exec, graph, cudaGraphInstantiateFlagUseNodePriority);
  cudaGraphDestroy(graph);
  if (ei != cudaSuccess) return fail(HGD_ECUDA, std::string("hgd_search: graph instantiate: ") + cudaGetErrorString(ei));
  w->graph_exec = exec;
  w->graph_key = key;
  HG_CUDA(cudaGraphLaunch(exec, st));
  return HGD_OK;
}

}  // extern "C"

namespace {

// Everything one batch enqueues on `st` (also the body a CUDA graph captures).
int enqueue_batch(hgd_graph* g, const hgd_search_args* a, Workspace* w, cudaStream_t st) {
  const uint64_t nq = a->nq;
  const uint32_t dim = static_cast<uint32_t>(g->dim);

  // ---- effective ef bound ----
  uint32_t ef_max = a->ef ? a->ef : a->ef_default;
  if (a->ef_per_query && !a->queries_on_device) {
    ef_max = 0;
    for (uint64_t i = 0; i < nq; ++i) {
      const uint32_t e = a->ef_per_query[i] ? a->ef_per_query[i] : a->ef_default;
      ef_max = std::max(ef_max, e);
    }
  }
  ef_max = std::max(ef_max, a->k);
  if (ef_max == 0) return fail(HGD_EINVAL, "hgd_search: ef is 0");
  if (a->k_per_query && !a->queries_on_device)
    for (uint64_t i = 0; i < nq; ++i)
      if (a->k_per_query[i] == 0 || a->k_per_query[i] > a->k)
        return fail(HGD_EINVAL, "hgd_search: per-query k must be in 1..k");

  // ---- inputs to the device ----
  const float* d_q = a->queries;
  const uint32_t* d_ef = a->ef_per_query;
  const uint32_t* d_k = a->k_per_query;
  if (!a->queries_on_device) {
    HG_CUDA(w->q.ensure(nq * dim * 4));
    HG_CUDA(cudaMemcpyAsync(w->q.p, a->queries, nq * dim * 4, cudaMemcpyHostToDevice, st));
    d_q = w->q.as<float>();
    if (a->ef_per_query) {
      HG_CUDA(w->efq.ensure(nq * 4));
      HG_CUDA(cudaMemcpyAsync(w->efq.p, a->ef_per_query, nq * 4, cudaMemcpyHostToDevice, st));
      d_ef = w->efq.as<uint32_t>();
    }
    if (a->k_per_query) {
      HG_CUDA(w->kq.ensure(nq * 4));
      HG_CUDA(cudaMemcpyAsync(w->kq.p, a->k_per_query, nq * 4, cudaMemcpyHostToDevice, st));
      d_k = w->kq.as<uint32_t>();
    }
  }
  // ---- filters -> id-space bitsets ----
  const uint32_t nw = static_cast<uint32_t>((g->n + 31) / 32) + 1;
  const int32_t* d_fsel = nullptr;
  const uint32_t* const* d_fptrs = nullptr;
  if (a->num_filters > 0) {
    uint64_t label_words = 0;
    for (uint32_t f = 0; f < a->num_filters; ++f)
      if (a->filters[f].label_space) label_words += (a->filters[f].num_bits + 63) / 64;
    HG_CUDA(w->fbits.ensure(static_cast<uint64_t>(a->num_filters) * nw * 4 + label_words * 8 + 64));
    uint32_t* idbits = w->fbits.as<uint32_t>();
    uint64_t* lw = reinterpret_cast<uint64_t*>(idbits + static_cast<uint64_t>(a->num_filters) * nw + 1);
    lw = reinterpret_cast<uint64_t*>((reinterpret_cast<uintptr_t>(lw) + 7) & ~uintptr_t(7));
    std::vector<const uint32_t*> ptrs(a->num_filters);
    for (uint32_t f = 0; f < a->num_filters; ++f) {
      const hgd_bitset& bs = a->filters[f];
      uint32_t* dst = idbits + static_cast<uint64_t>(f) * nw;
      ptrs[f] = dst;
      const uint64_t words64 = (bs.num_bits + 63) / 64;
      if (words64 && !bs.words) return fail(HGD_EINVAL, "hgd_search: null filter words");
      if (bs.label_space) {
        if (words64) HG_CUDA(cudaMemcpyAsync(lw, bs.words, words64 * 8, cudaMemcpyHostToDevice, st));
        HG_CUDA(hg::launch_translate_filter(lw, bs.num_bits, g->labels.as<uint64_t>(),
                                            static_cast<uint32_t>(g->n), dst, st));
        lw += words64;
      } else {
        // id space: copy min(num_bits, n) bits, the rest not allowed
        HG_CUDA(cudaMemsetAsync(dst, 0, nw * 4, st));
        const uint64_t bits = std::min<uint64_t>(bs.num_bits, g->n);
        const uint64_t full = bits / 64;
        if (full) HG_CUDA(cudaMemcpyAsync(dst, bs.words, full * 8, cudaMemcpyHostToDevice, st));
        if (bits % 64) {
          uint64_t last = bs.words[full] & ((1ull << (bits % 64)) - 1);
          // staged through pinned memory: the source must outlive the async copy
          HG_CUDA(w->pin_in.ensure(8));
          std::memcpy(w->pin_in.p, &last, 8);
          HG_CUDA(cudaMemcpyAsync(dst + 2 * full, w->pin_in.p, 8, cudaMemcpyHostToDevice, st));
          HG_CUDA(cudaStreamSynchronize(st));
        }
      }
    }
    HG_CUDA(w->fptrs.ensure(a->num_filters * sizeof(void*)));
    HG_CUDA(cudaMemcpyAsync(w->fptrs.p, ptrs.data(), a->num_filters * sizeof(void*), cudaMemcpyHostToDevice, st));
    d_fptrs = w->fptrs.as<const uint32_t* const>();
    HG_CUDA(w->fsel.ensure(nq * 4));
    if (a->filter_of_query) {
      for (uint64_t i = 0; i < nq; ++i)
        if (a->filter_of_query[i] >= static_cast<int32_t>(a->num_filters))
          return fail(HGD_EINVAL, "hgd_search: filter index out of range");
      HG_CUDA(cudaMemcpyAsync(w->fsel.p, a->filter_of_query, nq * 4, cudaMemcpyHostToDevice, st));
    } else {
      HG_CUDA(cudaMemsetAsync(w->fsel.p, 0, nq * 4, st));
    }
    d_fsel = w->fsel.as<int32_t>();
  }
  // ---- compressed-precision batches: restrictive filters go to the exact scan ----
  std::vector<uint32_t> r_qlist;
  std::vector<int32_t> r_fsel;
  std::vector<uint64_t> r_ones;  // per filter: rows it allows
  const uint8_t* d_skip = nullptr;
  if (a->filter_scan_mode > HGD_SCAN_EVERY_ROW) return fail(HGD_EINVAL, "hgd_search: unknown filter_scan_mode");
  if (a->precision != HGD_PREC_FP32 && a->filter_scan_permille && a->num_filters && !a->nres && !a->counters &&
      hg::bfm::supported(static_cast<uint32_t>(g->pd), a->k)) {
    std::vector<char> routed(a->num_filters, 0);
    r_ones.assign(a->num_filters, 0);
    bool any = false;
    for (uint32_t f = 0; f < a->num_filters; ++f) {
      const hgd_bitset& bs = a->filters[f];
      uint64_t ones = 0;
      const uint64_t words64 = (bs.num_bits + 63) / 64;
      for (uint64_t i = 0; i < words64; ++i) ones += static_cast<uint64_t>(__builtin_popcountll(bs.words[i]));
      r_ones[f] = ones;
      routed[f] = ones * 1000 <= static_cast<uint64_t>(a->filter_scan_permille) * g->n;
      any = any || routed[f];
    }
    if (any) {
      std::vector<uint8_t> skip(nq, 0);
      for (uint64_t q = 0; q < nq; ++q) {
        const int32_t f = a->filter_of_query ? a->filter_of_query[q] : 0;
        if (f >= 0 && routed[f]) {
          skip[q] = 1;
          r_qlist.push_back(static_cast<uint32_t>(q));
        }
      }
      // grouped by filter (the allowed-rows scan tiles the queries of one
      // filter together), in query order within a filter
      std::stable_sort(r_qlist.begin(), r_qlist.end(), [&](uint32_t x, uint32_t y) {
        return (a->filter_of_query ? a->filter_of_query[x] : 0) < (a->filter_of_query ? a->filter_of_query[y] : 0);
      });
      for (uint32_t q : r_qlist) r_fsel.push_back(a->filter_of_query ? a->filter_of_query[q] : 0);
      if (!r_qlist.empty()) {
        HG_CUDA(w->scan_route.ensure(nq));
        HG_CUDA(w->scan_qlist.ensure(r_qlist.size() * 4));
        HG_CUDA(w->scan_fsel.ensure(r_fsel.size() * 4));
        HG_CUDA(cudaMemcpyAsync(w->scan_route.p, skip.data(), nq, cudaMemcpyHostToDevice, st));
        HG_CUDA(cudaMemcpyAsync(w->scan_qlist.p, r_qlist.data(), r_qlist.size() * 4, cudaMemcpyHostToDevice, st));
        HG_CUDA(cudaMemcpyAsync(w->scan_fsel.p, r_fsel.data(), r_fsel.size() * 4, cudaMemcpyHostToDevice, st));
        d_skip = w->scan_route.as<uint8_t>();
      }
    }
  }
  // ---- cosine: 1/||q|| per query ----
  const float* d_inv = nullptr;
  if (g->metric == HGD_METRIC_COSINE) {
    HG_CUDA(w->inv.ensure(nq * 4));
    HG_CUDA(hg::launch_inv_norm(d_q, static_cast<uint32_t>(nq), dim, w->inv.as<float>(), st));
    d_inv = w->inv.as<float>();
  }
  // ---- outputs ----
  void* d_out = a->out;
  uint32_t* d_nres = a->nres;
  if (!a->out_on_device) {
    HG_CUDA(w->out.ensure(nq * a->k * 16));
    d_out = w->out.p;
    if (a->nres) {
      HG_CUDA(w->nres.ensure(nq * 4));
      d_nres = w->nres.as<uint32_t>();
    }
  }
  unsigned long long* d_cnt = nullptr;
  if (a->counters) {
    HG_CUDA(w->counters.ensure(nq * hg::kCounters * 8));
    d_cnt = w->counters.as<unsigned long long>();
  }

  // ---- launch shape ----
  hg::SearchParams P{};
  P.vecs = g->vecs.as<float>();
  P.l0 = g->l0.as<uint32_t>();
  P.up = g->up.as<uint32_t>();
  P.up_blk = g->up_blk.as<uint32_t>();
  P.labels = g->labels.as<uint64_t>();
  P.alive = g->alive.as<uint32_t>();
  P.n = static_cast<uint32_t>(g->n);
  P.pd = static_cast<uint32_t>(g->pd);
  P.dim = dim;
  P.M = static_cast<uint32_t>(g->M);
  P.M0 = static_cast<uint32_t>(2 * g->M);
  P.l0_stride = g->l0s;
  P.up_stride = g->ups;
  P.metric = g->metric;
  P.max_level = g->max_level;
  P.entry = g->entry;
  P.tagged = g->n < (1ull << 24) ? 1 : 0;
  P.dedup = g->dedup ? 1 : 0;
  P.deleted_any = g->num_deleted > 0 ? 1 : 0;
  P.order = g->order == HGD_ORDER_NEON ? 1 : 0;
  P.queries = d_q;
  P.nq = static_cast<uint32_t>(nq);
  P.efq = d_ef;
  P.kq = d_k;
  P.ef_all = a->ef;
  P.ef_default = a->ef_default;
  P.k_all = a->k;
  P.k_stride = a->k;
  P.fbits = d_fptrs;
  P.fsel = d_fsel;
  P.num_filters = a->num_filters;
  P.out = d_out;
  P.nres = d_nres;
  P.done = a->done_flags;
  P.counters = d_cnt;
  // ---- compressed traversal: FP16 / FP8 copies (built once) and the rerank pools ----
  const int prec = static_cast<int>(a->precision);
  if (prec != HGD_PREC_FP32) {
    // rows of the compressed copies: the smallest of 128, 256, 512, 1024 that holds dim
    const uint32_t pdc = g->dim <= 128 ? 128u : (g->dim <= 256 ? 256u : (g->dim <= 512 ? 512u : 1024u));
    if (g->dim > 1024) return fail(HGD_EINVAL, "hgd_search: FP16/FP8 traversal supports dim <= 1024");
    DBuf& vb = prec == HGD_PREC_FP16 ? g->v16 : g->v8;
    DBuf& va = prec == HGD_PREC_FP16 ? g->vaux16 : g->vaux8;
    bool& have = prec == HGD_PREC_FP16 ? g->has16 : g->has8;
    std::lock_guard<std::mutex> build_lock(g->mu);
    if (!have) {
      HG_CUDA(vb.ensure(g->n * pdc * (prec == HGD_PREC_FP16 ? 2 : 1)));
      HG_CUDA(va.ensure(g->n * 8));
      if (prec == HGD_PREC_FP8) HG_CUDA(g->vscale.ensure(g->n * 4));
      HG_CUDA(hg::launch_encode(g->vecs.as<float>(), static_cast<uint32_t>(g->n), static_cast<uint32_t>(g->pd), pdc,
                                prec, vb.p, prec == HGD_PREC_FP8 ? g->vscale.as<float>() : nullptr, va.as<float>(),
                                st));
      have = true;
    }
    P.vq = vb.p;
    P.vscale = prec == HGD_PREC_FP8 ? g->vscale.as<float>() : nullptr;
    P.vaux = va.as<float>();
    P.pdc = pdc;
    P.pool_stride = round_up(ef_max, 32);
    HG_CUDA(w->pool_ids.ensure(nq * P.pool_stride * 4));
    HG_CUDA(w->pool_n.ensure(nq * 4));
    P.pool_out = w->pool_ids.as<uint32_t>();
    P.pool_n = w->pool_n.as<uint32_t>();
    P.rerank_factor = a->rerank_factor;
  }
  auto launch = [&](const hg::SearchParams& B, int blocks, int wpb, cudaStream_t sb) {
    return prec == HGD_PREC_FP32 ? hg::launch_search(B, d_inv, blocks, wpb, sb)
                                 : hg::launch_search_approx(B, d_inv, blocks, wpb, sb);
  };

  if (a->cand_cap && (a->cand_cap < 128 || a->cand_cap % 32))
    return fail(HGD_EINVAL, "hgd_search: cand_cap must be a multiple of 32, >= 128");
  if (a->hash_slots && (a->hash_slots < 256 || (a->hash_slots & (a->hash_slots - 1))))
    return fail(HGD_EINVAL, "hgd_search: hash_slots must be a power of two >= 256");
  if (a->warps_per_block > 4) return fail(HGD_EINVAL, "hgd_search: warps_per_block must be 1..4");

  // ---- ef buckets: one launch shape per bucket, sized for its largest ef ----
  hg::BucketSpec spec{};
  {
    // bucket bounds 16, 32, 64, 96, 128, 192, 256, 384, 512, ... (x1.5 / x4/3 steps)
    static const uint32_t kHi[] = {16, 32, 64, 96, 128, 192, 256, 384, 512, 768, 1024};
    for (uint32_t hi : kHi) {
      if (spec.n == hg::kMaxBuckets - 1) break;
      spec.hi[spec.n++] = std::min(hi, ef_max);
      if (hi >= ef_max) break;
    }
    if (spec.hi[spec.n - 1] < ef_max) spec.hi[spec.n++] = ef_max;
  }
  struct Shape {
    uint32_t H, R, C;
    int wpb, blocks;
    uint32_t slot_base;
  };
  std::vector<hgd_tune_entry> tune;
  int launch_mode = HGD_LAUNCH_BUCKETS;
  {
    std::lock_guard<std::mutex> lk(g->ws_mu);
    tune = g->tune;
    launch_mode = g->launch_mode;
  }
  const bool single = launch_mode == HGD_LAUNCH_SINGLE && spec.n > 1;
  auto tuned = [&](uint32_t E) -> const hgd_tune_entry* {
    static const uint32_t kNominal[] = {16, 32, 64, 96, 128, 192, 256, 384, 512, 768, 1024};
    uint32_t nominal = 0;
    for (uint32_t hi : kNominal)
      if (hi >= E) {
        nominal = hi;
        break;
      }
    for (const auto& t : tune)
      if (t.precision == a->precision && t.ef_hi == nominal) return &t;
    return nullptr;
  };
  std::vector<Shape> shapes(spec.n);
  uint64_t slots_total = 0;
  for (uint32_t b = 0; b < spec.n; ++b) {
    Shape& sh = shapes[b];
    const uint32_t E = spec.hi[b];
    const hgd_tune_entry* t = tuned(E);
    sh.R = round_up(E, 32);
    sh.C = a->cand_cap ? a->cand_cap
                       : (t && t->cand_cap ? t->cand_cap : std::max<uint32_t>(128, round_up(E + 32, 32)));
    sh.H = a->hash_slots ? a->hash_slots
                         : (t && t->hash_slots ? t->hash_slots : (E <= 32 ? 1024u : (E <= 512 ? 2048u : 4096u)));
    const uint32_t wbytes = hg::warp_smem_bytes(sh.H, sh.R, sh.C);
    sh.wpb = static_cast<int>(std::min<uint32_t>(4, (227u * 1024u) / wbytes));
    const uint32_t want_wpb = a->warps_per_block ? a->warps_per_block : (t ? t->warps_per_block : 0u);
    if (want_wpb) sh.wpb = std::min<int>(sh.wpb, static_cast<int>(want_wpb));
    if (sh.wpb < 1) return fail(HGD_EINVAL, "hgd_search: ef too large for shared memory");
    const int occ = prec == HGD_PREC_FP32
                        ? hg::search_occupancy(static_cast<uint32_t>(g->pd), g->metric, P.order, sh.wpb, sh.H, sh.R,
                                               sh.C)
                        : hg::occupancy_approx(P.pdc, g->metric, prec, P.order, sh.wpb,
                                               static_cast<size_t>(sh.wpb) * hg::warp_smem_bytes(sh.H, sh.R, sh.C));
    if (occ < 1) return fail(HGD_ECUDA, "hgd_search: the search kernel cannot be resident with this shape");
    const uint64_t want = (nq + sh.wpb - 1) / sh.wpb;
    sh.blocks = static_cast<int>(std::min<uint64_t>(want, static_cast<uint64_t>(g->sms) * occ));
    sh.slot_base = static_cast<uint32_t>(slots_total);
    if (!single || b + 1 == spec.n) slots_total += static_cast<uint64_t>(sh.blocks) * sh.wpb;
  }
  if (single) shapes.back().slot_base = 0;
  // shared scratch: spill pools and visited bitmaps acquired per query
  const uint64_t bw = (g->n + 31) / 32 + 1;
  const uint64_t pool_cap = a->pool_cap ? std::max<uint64_t>(a->pool_cap, 32)
                                        : std::min<uint64_t>(std::max<uint64_t>(g->n, 1), 8192);
  // Bitmaps and first-tier pools: one per warp that can be resident at once
  // (every warp keeps at least the smallest shape's shared memory), so
  // acquisition does not fail unless a memory cap binds.  The first tier
  // holds 8K keys; queries whose candidate queue outgrows it (filtered
  // searches: every visited node enters the queue until ef eligible results
  // are found) move to a second tier of up to 2^18 keys.
  const uint64_t resident = static_cast<uint64_t>(g->sms) * std::min<uint64_t>(64, (228u * 1024u) / hg::warp_smem_bytes(1024, 32, 128));
  const uint32_t pool_slots = static_cast<uint32_t>(
      std::max<uint64_t>(1, std::min<uint64_t>({slots_total, resident, hg::kPoolBytesCap / (pool_cap * 8)})));
  const uint32_t bm_slots = static_cast<uint32_t>(
      std::max<uint64_t>(1, std::min<uint64_t>({slots_total, resident, hg::kBitmapBytesCap / (bw * 4)})));
  const uint64_t big_cap = a->pool_cap ? 0 : std::min<uint64_t>(std::max<uint64_t>(g->n, 1), uint64_t{1} << 18);
  const uint32_t big_slots = big_cap <= pool_cap ? 0u
                             : static_cast<uint32_t>(std::max<uint64_t>(
                                   1, std::min<uint64_t>({slots_total, resident, hg::kBigPoolBytesCap / (big_cap * 8)})));
  HG_CUDA(w->pool.ensure(pool_slots * pool_cap * 8));
  HG_CUDA(w->bitmaps.ensure(bm_slots * bw * 4));
  if (big_slots) HG_CUDA(w->pool_t2.ensure(big_slots * big_cap * 8));
  HG_CUDA(w->owners.ensure((pool_slots + bm_slots + big_slots) * 4));
  HG_CUDA(w->work.ensure(64 * 4));
  HG_CUDA(w->ovf_list.ensure(nq * 4));
  HG_CUDA(w->lists.ensure(static_cast<uint64_t>(spec.n) * nq * 4));
  HG_CUDA(cudaMemsetAsync(w->work.p, 0, 64 * 4, st));
  HG_CUDA(cudaMemsetAsync(w->owners.p, 0, (pool_slots + bm_slots + big_slots) * 4, st));
  uint32_t* work = w->work.as<uint32_t>();  // [1] overflow count [2] rerun work [4] error
                                            // [8+b] bucket work  [32+b] bucket size
  P.pool = w->pool.as<uint64_t>();
  P.pool_cap = pool_cap;
  P.pool_owner = w->owners.as<uint32_t>();
  P.pool_slots = pool_slots;
  P.bitmaps = w->bitmaps.as<uint32_t>();
  P.bitmap_words = bw;
  P.bm_owner = w->owners.as<uint32_t>() + pool_slots;
  P.bm_slots = bm_slots;
  P.big_pool = big_slots ? w->pool_t2.as<uint64_t>() : nullptr;
  P.big_cap = big_cap;
  P.big_owner = big_slots ? w->owners.as<uint32_t>() + pool_slots + bm_slots : nullptr;
  P.big_slots = big_slots;
  P.ovf_count = work + 1;
  P.ovf_list = w->ovf_list.as<uint32_t>();
  P.err = work + 4;
  {
    cudaError_t e = hg::launch_bucket(d_ef, d_k, static_cast<uint32_t>(nq), a->ef, a->ef_default, a->k, spec,
                                      work + 32, w->lists.as<uint32_t>(), st, d_skip);
    if (e != cudaSuccess) return fail(HGD_ECUDA, std::string("bucket kernel launch: ") + cudaGetErrorString(e));
  }
  // fork: each bucket on its own stream, largest ef first, joined back into st
  if (w->aux.size() < spec.n) {
    if (!w->ev_fork) HG_CUDA(cudaEventCreateWithFlags(&w->ev_fork, cudaEventDisableTiming));
    int least = 0, greatest = 0;
    HG_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    while (w->aux.size() < spec.n) {
      cudaStream_t s2 = nullptr;
      cudaEvent_t e2 = nullptr;
      // larger-ef buckets get higher priority: their blocks take the SMs first
      // and the short queries fill in (also inside a captured graph)
      const int b = static_cast<int>(w->aux.size());
      const int prio = std::max(greatest, least - b / 2);
      HG_CUDA(cudaStreamCreateWithPriority(&s2, cudaStreamNonBlocking, prio));
      HG_CUDA(cudaEventCreateWithFlags(&e2, cudaEventDisableTiming));
      w->aux.push_back(s2);
      w->ev_join.push_back(e2);
    }
  }
  // routed queries: the exact scan on the workspace's scan stream, concurrent
  // with the walk, joined before the results leave
  const bool scanning = !r_qlist.empty();
  if (scanning) {
    hg::bfm::Rows rows{g->vecs.as<float>(), g->labels.as<uint64_t>(), static_cast<uint32_t>(g->n),
                       static_cast<uint32_t>(g->pd), static_cast<uint32_t>(g->pd), g->metric,
                       g->order == HGD_ORDER_NEON ? 1 : 0};
    {
      std::lock_guard<std::mutex> build_lock(g->mu);
      if (!g->scan) {
        std::string err;
        if (hg::bfm::store_create(rows, st, &g->scan, &err) != cudaSuccess) return fail(HGD_ECUDA, err);
      }
    }
    if (!w->scan_sc) w->scan_sc = hg::bfm::scratch_new();
    if (!w->scan_stream) {
      HG_CUDA(cudaStreamCreateWithFlags(&w->scan_stream, cudaStreamNonBlocking));
      HG_CUDA(cudaEventCreateWithFlags(&w->scan_fork, cudaEventDisableTiming));
      HG_CUDA(cudaEventCreateWithFlags(&w->scan_join, cudaEventDisableTiming));
    }
    HG_CUDA(cudaEventRecord(w->scan_fork, st));
    HG_CUDA(cudaStreamWaitEvent(w->scan_stream, w->scan_fork, 0));
    hg::bfm::RoutedArgs ra{};
    ra.queries = d_q;
    ra.inv = d_inv;
    ra.qlist = w->scan_qlist.as<uint32_t>();
    ra.fsel = w->scan_fsel.as<int32_t>();
    ra.allow_tab = d_fptrs;
    ra.alive = g->alive.as<uint32_t>();
    ra.n_r = static_cast<uint32_t>(r_qlist.size());
    ra.dim = dim;
    ra.k_stride = a->k;
    ra.kq = d_k;
    ra.out = d_out;
    ra.done = a->done_flags;
    ra.h_fsel = r_fsel.data();
    ra.h_ones = r_ones.data();
    ra.mode = static_cast<int>(a->filter_scan_mode);
    std::string err;
    if (hg::bfm::search_routed(g->scan, rows, ra, w->scan_sc, w->scan_stream, &err) != cudaSuccess)
      return fail(HGD_ECUDA, err);
    HG_CUDA(cudaEventRecord(w->scan_join, w->scan_stream));
  }
  // several warps per query (compressed rows of 128 elements): one CTA per
  // query, every bucket largest ef first; overflows go to the rerun pass
  const bool wide = a->warps_per_query >= 4 && prec != HGD_PREC_FP32 && P.pdc == 128 && g->n > 0 &&
                    g->n < (1ull << 24) && P.M0 <= 32 && a->counters == nullptr;
  // one warp per query, a beam search over several lists per step with
  // tensor-core distances (compressed rows of 128 elements)
  const bool beamwalk = !wide && a->lists_per_step >= 1 && prec != HGD_PREC_FP32 && P.pdc == 128 && g->n > 0 &&
                        g->n < (1ull << 24) && P.M0 <= 32;
  if (beamwalk) {
    // filters or deletes: the variant that keeps a separate result list
    const bool filt = a->num_filters > 0 || g->num_deleted > 0;
    const int wpb = 4;
    // one launch over every query with the largest bucket's shape, or --
    // per-query ef spread over several buckets -- one launch per bucket with
    // its own shape (the beam and hash of a large ef would otherwise cut the
    // occupancy of every query), concurrent on the workspace's forked
    // streams, larger ef first.  A query walks the same in either: its hash
    // size and beam capacity follow its own ef.
    const bool per_bucket = a->ef_per_query != nullptr && spec.n > 1;
    if (per_bucket) HG_CUDA(cudaEventRecord(w->ev_fork, st));
    for (int b = per_bucket ? static_cast<int>(spec.n) - 1 : 0; b >= 0; --b) {
      const uint32_t hi = per_bucket ? spec.hi[b] : ef_max;
      hg::SearchParams B = P;
      B.R = round_up(hi, 32);
      // visited hash slots: each query uses the size its own ef calls for
      // (beam_hash_slots); the launch reserves the largest
      B.H = hg::beam_hash_slots(hi);
      B.lists_per_step = std::min<uint32_t>(a->lists_per_step, hg::kBeamMaxE);
      B.slot_base = 0;
      if (per_bucket) {
        B.nq_dev = work + 32 + b;
        B.qidx = w->lists.as<uint32_t>() + static_cast<uint64_t>(b) * nq;
        B.work = work + 8 + b;
      } else {
        B.qidx = w->lists.as<uint32_t>();
        B.lpt_sizes = work + 32;
        B.lpt_buckets = spec.n;
        B.lpt_stride = static_cast<uint32_t>(nq);
        B.work = work + 8;
      }
      const size_t smem = static_cast<size_t>(wpb) * hg::beam_warp_bytes(B.H, B.R, filt);
      if (smem > 227u * 1024u) return fail(HGD_EINVAL, "hgd_search: ef too large for the beam walk's shared memory");
      const int occ = hg::occupancy_beam(g->metric, prec, P.order, wpb, smem, filt);
      if (occ < 1) return fail(HGD_ECUDA, "hgd_search: the beam kernel cannot be resident");
      const uint64_t want = (nq + wpb - 1) / wpb;
      const int blocks = static_cast<int>(std::min<uint64_t>(want, static_cast<uint64_t>(g->sms) * occ));
      cudaStream_t sb = st;
      if (per_bucket) {
        sb = w->aux[b];
        HG_CUDA(cudaStreamWaitEvent(sb, w->ev_fork, 0));
      }
      cudaError_t e = hg::launch_search_beam(B, d_inv, blocks, wpb, filt, sb);
      if (e != cudaSuccess) return fail(HGD_ECUDA, std::string("beam kernel launch: ") + cudaGetErrorString(e));
      if (per_bucket) HG_CUDA(cudaEventRecord(w->ev_join[b], sb));
    }
    if (per_bucket)
      for (uint32_t b = 0; b < spec.n; ++b) HG_CUDA(cudaStreamWaitEvent(st, w->ev_join[b], 0));
  } else if (wide) {
    hg::SearchParams B = P;
    B.R = round_up(ef_max, 32);
    B.qidx = w->lists.as<uint32_t>();
    B.lpt_sizes = work + 32;
    B.lpt_buckets = spec.n;
    B.lpt_stride = static_cast<uint32_t>(nq);
    B.work = work + 8;
    B.slot_base = 0;
    const int occ = hg::occupancy_wide(g->metric, prec, P.order, B.R);
    if (occ < 1) return fail(HGD_ECUDA, "hgd_search: the several-warps kernel cannot be resident");
    const int blocks = static_cast<int>(std::min<uint64_t>(nq, static_cast<uint64_t>(g->sms) * occ));
    cudaError_t e = hg::launch_search_wide(B, d_inv, blocks, st);
    if (e != cudaSuccess) return fail(HGD_ECUDA, std::string("search kernel launch: ") + cudaGetErrorString(e));
  } else if (single) {
    // one persistent launch, the largest bucket's shape, every query
    const Shape& sh = shapes.back();
    hg::SearchParams B = P;
    B.H = sh.H;
    B.R = sh.R;
    B.C = sh.C;
    B.qidx = w->lists.as<uint32_t>();
    B.lpt_sizes = work + 32;
    B.lpt_buckets = spec.n;
    B.lpt_stride = static_cast<uint32_t>(nq);
    B.work = work + 8;
    B.slot_base = 0;
    cudaError_t e = launch(B, sh.blocks, sh.wpb, st);
    if (e != cudaSuccess) return fail(HGD_ECUDA, std::string("search kernel launch: ") + cudaGetErrorString(e));
  } else {
  HG_CUDA(cudaEventRecord(w->ev_fork, st));
  for (int b = static_cast<int>(spec.n) - 1; b >= 0; --b) {
    const Shape& sh = shapes[b];
    cudaStream_t sb = w->aux[b];
    HG_CUDA(cudaStreamWaitEvent(sb, w->ev_fork, 0));
    hg::SearchParams B = P;
    B.H = sh.H;
    B.R = sh.R;
    B.C = sh.C;
    B.nq_dev = work + 32 + b;
    B.qidx = w->lists.as<uint32_t>() + static_cast<uint64_t>(b) * nq;
    B.work = work + 8 + b;
    B.slot_base = sh.slot_base;
    cudaError_t e = launch(B, sh.blocks, sh.wpb, sb);
    if (e != cudaSuccess) return fail(HGD_ECUDA, std::string("search kernel launch: ") + cudaGetErrorString(e));
    HG_CUDA(cudaEventRecord(w->ev_join[b], sb));
  }
  for (uint32_t b = 0; b < spec.n; ++b) HG_CUDA(cudaStreamWaitEvent(st, w->ev_join[b], 0));
  }
  // ---- rerun of queries that ran out of spill pool or bitmap: per-warp pool of n keys ----
  {
    const uint64_t rerun_slots = 32;
    const uint64_t rerun_cap = std::max<uint64_t>(g->n, 1);
    HG_CUDA(w->pool_big.ensure(rerun_slots * rerun_cap * 8));
    HG_CUDA(w->bitmaps_big.ensure(rerun_slots * bw * 4));
    hg::SearchParams B = P;
    B.R = round_up(ef_max, 32);
    B.C = std::max<uint32_t>(128, round_up(ef_max + 32, 32));
    B.H = 4096;
    B.nq_dev = work + 1;
    B.qidx = w->ovf_list.as<uint32_t>();
    B.work = work + 2;
    B.pool = w->pool_big.as<uint64_t>();
    B.pool_cap = rerun_cap;
    B.pool_owner = nullptr;
    B.big_owner = nullptr;
    B.big_pool = nullptr;
    B.big_slots = 0;
    B.bitmaps = w->bitmaps_big.as<uint32_t>();
    B.bm_owner = nullptr;
    B.slot_base = 0;
    B.ovf_count = work + 3;  // cannot overflow: cap = n, one bitmap per warp
    B.rerun = 1;
    const uint32_t wb = hg::warp_smem_bytes(B.H, B.R, B.C);
    if (wb > 227u * 1024u) return fail(HGD_EINVAL, "hgd_search: ef too large for shared memory");
    cudaError_t e = launch(B, static_cast<int>(rerun_slots), 1, st);
    if (e != cudaSuccess) return fail(HGD_ECUDA, std::string("rerun kernel launch: ") + cudaGetErrorString(e));
  }
  if (scanning) HG_CUDA(cudaStreamWaitEvent(st, w->scan_join, 0));
  // ---- results back ----
  if (!a->out_on_device) {
    HG_CUDA(cudaMemcpyAsync(a->out, d_out, nq * a->k * 16, cudaMemcpyDeviceToHost, st));
    if (a->nres) HG_CUDA(cudaMemcpyAsync(a->nres, d_nres, nq * 4, cudaMemcpyDeviceToHost, st));
  }
  if (a->counters)
    HG_CUDA(cudaMemcpyAsync(a->counters, d_cnt, nq * hg::kCounters * 8, cudaMemcpyDeviceToHost, st));
  HG_CUDA(w->pin_out.ensure(8));
  HG_CUDA(cudaMemcpyAsync(w->pin_out.p, w->work.as<uint32_t>() + 4, 4, cudaMemcpyDeviceToHost, st));
  if (a->synchronize || a->counters) {
    HG_CUDA(cudaStreamSynchronize(st));
    if (*static_cast<uint32_t*>(w->pin_out.p) != 0)
      return fail(HGD_EINVAL, "hgd_search: a per-query ef or k exceeds the bound given for this batch");
  }
  return HGD_OK;
}

}  // namespace

extern "C" {

int hgd_graph_set_tuning(hgd_graph* g, const hgd_tune_entry* entries, uint32_t n) {
  if (!g || (n && !entries)) return fail(HGD_EINVAL, "hgd_graph_set_tuning: null argument");
  for (uint32_t i = 0; i < n; ++i) {
    const hgd_tune_entry& e = entries[i];
    if (e.precision > HGD_PREC_FP8 || (e.hash_slots && (e.hash_slots < 256 || (e.hash_slots & (e.hash_slots - 1)))) ||
        (e.cand_cap && (e.cand_cap < 128 || e.cand_cap % 32)) || e.warps_per_block > 4)
      return fail(HGD_EINVAL, "hgd_graph_set_tuning: bad entry");
  }
  std::lock_guard<std::mutex> lk(g->ws_mu);
  g->tune.assign(entries, entries + n);
  ++g->tune_version;
  return HGD_OK;
}

int hgd_graph_set_launch_mode(hgd_graph* g, int mode) {
  if (!g || (mode != HGD_LAUNCH_BUCKETS && mode != HGD_LAUNCH_SINGLE))
    return fail(HGD_EINVAL, "hgd_graph_set_launch_mode: bad argument");
  std::lock_guard<std::mutex> lk(g->ws_mu);
  g->launch_mode = mode;
  ++g->tune_version;
  return HGD_OK;
}

uint32_t hgd_shape_smem_bytes(uint32_t hash_slots, uint32_t ef_hi, uint32_t cand_cap) {
  return hg::warp_smem_bytes(hash_slots, round_up(ef_hi, 32), cand_cap);
}

int hgd_graph_device_info(const hgd_graph* g, char* name, uint32_t name_cap, uint32_t* sms) {
  if (!g) return fail(HGD_EINVAL, "hgd_graph_device_info: null graph");
  cudaDeviceProp p{};
  HG_CUDA(cudaGetDeviceProperties(&p, g->device));
  if (name && name_cap) {
    std::strncpy(name, p.name, name_cap - 1);
    name[name_cap - 1] = 0;
  }
  if (sms) *sms = static_cast<uint32_t>(p.multiProcessorCount);
  return HGD_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free batch over an uploaded graph (hg_index_search_batch_noalloc)
// ---------------------------------------------------------------------------
namespace hg {
uint32_t noalloc_max_nodes();
uint32_t noalloc_max_queries();
uint32_t noalloc_max_ef();
cudaError_t launch_search_noalloc(SearchParams P, int device, bool cosine, cudaStream_t st);

// Queries (nq x dim float32) and out (nq x k records) are device pointers;
// one ef for the batch (0: ef_default), no filters.  Nothing is allocated:
// scratch comes from the library's static device array, so batches that
// overlap on the GPU race on it.  Returns an HGD_* status.
int search_noalloc(hgd_graph* g, const float* d_queries, uint64_t nq, uint32_t k, uint32_t ef, uint32_t ef_default,
                   void* d_out, void* stream) {
  if (!g || !d_queries || !d_out) return fail(HGD_EINVAL, "search (no-alloc): null pointer");
  if (k == 0) return fail(HGD_EINVAL, "search (no-alloc): k must be > 0");
  if (nq == 0) return HGD_OK;
  if (nq > noalloc_max_queries())
    return fail(HGD_EINVAL, "search (no-alloc): at most " + std::to_string(noalloc_max_queries()) +
                                " queries per call");
  if (g->n > noalloc_max_nodes())
    return fail(HGD_EINVAL, "search (no-alloc): graphs above " + std::to_string(noalloc_max_nodes()) +
                                " nodes need the allocating entry points");
  uint32_t e = ef ? ef : ef_default;
  e = std::max(e, k);
  if (e == 0 || e > noalloc_max_ef())
    return fail(HGD_EINVAL, "search (no-alloc): ef (after max(ef, k)) must be 1.." +
                                std::to_string(noalloc_max_ef()));
  HG_CUDA(cudaSetDevice(g->device));
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : g->stream;
  hg::SearchParams P{};
  P.vecs = g->vecs.as<float>();
  P.l0 = g->l0.as<uint32_t>();
  P.up = g->up.as<uint32_t>();
  P.up_blk = g->up_blk.as<uint32_t>();
  P.labels = g->labels.as<uint64_t>();
  P.alive = g->alive.as<uint32_t>();
  P.n = static_cast<uint32_t>(g->n);
  P.pd = static_cast<uint32_t>(g->pd);
  P.dim = static_cast<uint32_t>(g->dim);
  P.M = static_cast<uint32_t>(g->M);
  P.M0 = static_cast<uint32_t>(2 * g->M);
  P.l0_stride = g->l0s;
  P.up_stride = g->ups;
  P.metric = g->metric;
  P.max_level = g->max_level;
  P.entry = g->entry;
  P.tagged = g->n < (1ull << 24) ? 1 : 0;
  P.dedup = g->dedup ? 1 : 0;
  P.deleted_any = g->num_deleted > 0 ? 1 : 0;
  P.order = g->order == HGD_ORDER_NEON ? 1 : 0;
  P.queries = d_queries;
  P.nq = static_cast<uint32_t>(nq);
  P.ef_all = e;
  P.ef_default = e;
  P.k_all = k;
  P.k_stride = k;
  P.out = d_out;
  P.R = round_up(e, 32);
  P.C = std::max<uint32_t>(128, next_pow2(e + 32));
  P.H = 4096;
  const cudaError_t ce = hg::launch_search_noalloc(P, g->device, g->metric == HGD_METRIC_COSINE, st);
  if (ce != cudaSuccess) return fail(HGD_ECUDA, std::string("search (no-alloc): ") + cudaGetErrorString(ce));
  return HGD_OK;
}
}  // namespace hg
