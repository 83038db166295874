// tune.cpp -- launch-shape autotuner for the batched query kernels.
//
// The query kernel's shape per ef bucket -- visited-hash slots per warp,
// candidate-head capacity per warp (the on-chip part of the candidate heap)
// and warps per block -- trades shared memory (and so resident warps) against
// spills to the global bitmap / pool.  The best point depends on the graph
// (n, degree, dimension), the precision and the GPU, so it is measured: for
// each bucket up to ef_max, every feasible shape of a small grid runs a
// sample batch whose queries all carry the bucket's ef, timed with CUDA
// events after a warm-up, and the fastest shape is kept.  Given per-query ef
// for the sample, the buckets run concurrently as in a real mixed batch, so
// the table is found on the whole batch's time instead: first one shape for
// every bucket, then one bucket at a time, largest first.  The table goes to
// the device mirror (hgd_graph_set_tuning) and to JSON for reuse.  No
// counterpart in the reference (its search runs one query per CPU thread).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <limits>
#include <shared_mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "graph.hpp"

namespace hnsw::gb {

namespace {

constexpr uint32_t kBuckets[] = {16, 32, 64, 96, 128, 192, 256, 384, 512, 768, 1024};
constexpr uint32_t kSmemPerBlock = 227u * 1024u;

struct DevMem {
  void* p = nullptr;
  ~DevMem() {
    if (p) cudaFree(p);
  }
};

void cuda_ok(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw std::runtime_error(std::string("autotune: ") + what + ": " + cudaGetErrorString(e));
}

uint32_t round_up32(uint32_t v) { return (v + 31u) / 32u * 32u; }

}  // namespace

std::string autotune(Index::Impl& im, const float* queries, size_t nq, uint32_t k, uint32_t ef_max, int precision,
                     const uint32_t* ef_per_query) {
  if (!queries || nq == 0) throw std::invalid_argument("autotune: no sample queries");
  if (k == 0) throw std::invalid_argument("autotune: k must be > 0");
  if (precision < 0 || precision > 2) throw std::invalid_argument("autotune: precision must be 0, 1 or 2");
  std::shared_lock<std::shared_mutex> lk(im.api_mutex);
  if (im.count == 0) throw std::invalid_argument("autotune: empty index");
  hgd_graph* g = im.device_graph();
  cuda_ok(cudaSetDevice(im.device), "device");
  const size_t dim = im.dim;
  DevMem dq, dout, def;
  cuda_ok(cudaMalloc(&dq.p, nq * dim * 4), "alloc");
  cuda_ok(cudaMemcpy(dq.p, queries, nq * dim * 4, cudaMemcpyHostToDevice), "copy");
  uint32_t mix_max = 0;
  if (ef_per_query) {
    for (size_t i = 0; i < nq; ++i) mix_max = std::max(mix_max, std::max(ef_per_query[i], k));
    if (mix_max == 0 || mix_max > 1024) throw std::invalid_argument("autotune: per-query ef must be in 1..1024");
    cuda_ok(cudaMalloc(&def.p, nq * 4), "alloc");
    cuda_ok(cudaMemcpy(def.p, ef_per_query, nq * 4, cudaMemcpyHostToDevice), "copy");
  }
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cuda_ok(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "stream");
  cuda_ok(cudaEventCreate(&e0), "event");
  cuda_ok(cudaEventCreate(&e1), "event");
  struct Guard {
    cudaStream_t s;
    cudaEvent_t a, b;
    ~Guard() {
      cudaStreamDestroy(s);
      cudaEventDestroy(a);
      cudaEventDestroy(b);
    }
  } guard{st, e0, e1};

  // time one shape (0 fields = the default rule): microseconds per query
  auto time_shape = [&](uint32_t ef, uint32_t kk, uint32_t H, uint32_t C, uint32_t wpb) -> double {
    hgd_search_args a{};
    if (def.p) a.ef_per_query = static_cast<const uint32_t*>(def.p);
    a.queries = static_cast<const float*>(dq.p);
    a.queries_on_device = 1;
    a.out_on_device = 1;
    a.nq = nq;
    a.k = kk;
    a.ef = ef;
    a.ef_default = ef;
    a.precision = static_cast<uint32_t>(precision);
    a.out = dout.p;
    a.stream = st;
    a.hash_slots = H;
    a.cand_cap = C;
    a.warps_per_block = wpb;
    double best = std::numeric_limits<double>::infinity();
    for (int rep = 0; rep < 3; ++rep) {
      cuda_ok(cudaEventRecord(e0, st), "event");
      const int rc = hgd_search(g, &a);
      if (rc != HGD_OK) throw std::runtime_error(std::string("autotune: search: ") + hgd_last_error());
      cuda_ok(cudaEventRecord(e1, st), "event");
      cuda_ok(cudaEventSynchronize(e1), "sync");
      float ms = 0.0f;
      cuda_ok(cudaEventElapsedTime(&ms, e0, e1), "timing");
      if (rep > 0) best = std::min(best, static_cast<double>(ms));  // rep 0 warms up
    }
    return best * 1e3 / static_cast<double>(nq);
  };

  int launch_mode = im.launch_mode;
  std::vector<hgd_tune_entry> table;
  for (const auto& t : im.tuning)
    if (static_cast<int>(t.precision) != precision) table.push_back(t);  // keep other precisions
  std::string rows;
  // the default rule runs while the table is measured
  {
    std::vector<hgd_tune_entry> others = table;
    hgd_graph_set_tuning(g, others.data(), static_cast<uint32_t>(others.size()));
  }
  if (ef_per_query) {
    // ---- mixed batch: coordinate descent over the buckets present ----
    std::vector<uint32_t> present;
    for (size_t bi = 0; bi < sizeof(kBuckets) / sizeof(kBuckets[0]); ++bi) {
      const uint32_t E = kBuckets[bi];
      const uint32_t lo = bi == 0 ? 0u : kBuckets[bi - 1];
      bool any = false;
      for (size_t i = 0; i < nq && !any; ++i) {
        const uint32_t e = std::max(ef_per_query[i], k);
        any = e > lo && e <= E;
      }
      if (any) present.push_back(E);
    }
    std::vector<hgd_tune_entry> mine;
    for (uint32_t E : present) mine.push_back(hgd_tune_entry{static_cast<uint32_t>(precision), E, 0, 0, 0, 0});
    auto install = [&]() {
      std::vector<hgd_tune_entry> all = table;
      all.insert(all.end(), mine.begin(), mine.end());
      if (hgd_graph_set_tuning(g, all.data(), static_cast<uint32_t>(all.size())) != HGD_OK)
        throw std::runtime_error(std::string("autotune: ") + hgd_last_error());
    };
    cuda_ok(cudaMalloc(&dout.p, nq * k * 16), "alloc");
    hgd_graph_set_launch_mode(g, HGD_LAUNCH_BUCKETS);
    install();
    const double t_default = time_shape(mix_max, k, 0, 0, 0);
    double best = t_default;
    // phase 1: one shape for every bucket (the buckets share the SMs, so
    // shrinking all of them together is what frees room for more warps)
    {
      std::vector<hgd_tune_entry> keep = mine;
      for (uint32_t H : {512u, 1024u, 2048u, 4096u})
        for (int half = 0; half < 2; ++half)
          for (uint32_t wpb : {1u, 2u, 4u}) {
            for (size_t bi = 0; bi < present.size(); ++bi) {
              const uint32_t E = present[bi];
              const uint32_t C = std::max<uint32_t>(128, round_up32((half ? E / 2 : E) + 32));
              mine[bi] = static_cast<uint64_t>(wpb) * hgd_shape_smem_bytes(H, E, C) <= kSmemPerBlock
                             ? hgd_tune_entry{static_cast<uint32_t>(precision), E, H, C, wpb, 0}
                             : hgd_tune_entry{static_cast<uint32_t>(precision), E, 0, 0, 0, 0};
            }
            install();
            const double t = time_shape(mix_max, k, 0, 0, 0);
            if (t < best * 0.995) {
              best = t;
              keep = mine;
            }
          }
      mine = keep;
      install();
    }
    // phase 2: one bucket at a time
    for (int pass = 0; pass < 1; ++pass) {
      for (size_t bi = present.size(); bi-- > 0;) {
        const uint32_t E = present[bi];
        const uint32_t c_full = std::max<uint32_t>(128, round_up32(E + 32));
        const uint32_t c_half = std::max<uint32_t>(128, round_up32(E / 2 + 32));
        hgd_tune_entry keep = mine[bi];
        for (uint32_t H : {512u, 1024u, 2048u, 4096u})
          for (uint32_t C : {c_full, c_half}) {
            if (C == c_half && c_half == c_full) continue;
            for (uint32_t wpb : {1u, 2u, 4u}) {
              if (static_cast<uint64_t>(wpb) * hgd_shape_smem_bytes(H, E, C) > kSmemPerBlock) continue;
              mine[bi] = hgd_tune_entry{static_cast<uint32_t>(precision), E, H, C, wpb, 0};
              install();
              const double t = time_shape(mix_max, k, 0, 0, 0);
              if (t < best * 0.995) {
                best = t;
                keep = mine[bi];
              }
            }
          }
        mine[bi] = keep;
        install();
      }
    }
    // the other launch mode: one largest-ef-first launch with the top
    // bucket's shape (the only entry it reads)
    int mode = HGD_LAUNCH_BUCKETS;
    {
      const std::vector<hgd_tune_entry> bucket_table = mine;
      hgd_graph_set_launch_mode(g, HGD_LAUNCH_SINGLE);
      const size_t top = present.size() - 1;
      const uint32_t E = present[top];
      const uint32_t c_full = std::max<uint32_t>(128, round_up32(E + 32));
      const uint32_t c_half = std::max<uint32_t>(128, round_up32(E / 2 + 32));
      double best_single = std::numeric_limits<double>::infinity();
      hgd_tune_entry keep = mine[top];
      for (uint32_t H : {512u, 1024u, 2048u, 4096u})
        for (uint32_t C : {c_full, c_half}) {
          if (C == c_half && c_half == c_full) continue;
          for (uint32_t wpb : {1u, 2u, 4u}) {
            if (static_cast<uint64_t>(wpb) * hgd_shape_smem_bytes(H, E, C) > kSmemPerBlock) continue;
            mine[top] = hgd_tune_entry{static_cast<uint32_t>(precision), E, H, C, wpb, 0};
            install();
            const double t = time_shape(mix_max, k, 0, 0, 0);
            if (t < best_single) {
              best_single = t;
              keep = mine[top];
            }
          }
        }
      if (best_single < best * 0.995) {
        mode = HGD_LAUNCH_SINGLE;
        best = best_single;
        mine[top] = keep;
      } else {
        mine = bucket_table;
        hgd_graph_set_launch_mode(g, HGD_LAUNCH_BUCKETS);
      }
      install();
    }
    launch_mode = mode;
    for (size_t bi = 0; bi < present.size(); ++bi) {
      const hgd_tune_entry& e = mine[bi];
      char buf[256];
      std::snprintf(buf, sizeof buf,
                    "%s    {\"precision\": %d, \"ef_hi\": %u, \"hash_slots\": %u, \"cand_cap\": %u, "
                    "\"warps_per_block\": %u, \"us_per_query\": %.4f, \"default_us_per_query\": %.4f}",
                    rows.empty() ? "" : ",\n", precision, e.ef_hi, e.hash_slots, e.cand_cap, e.warps_per_block, best,
                    t_default);
      rows += buf;
    }
    table.insert(table.end(), mine.begin(), mine.end());
  }
  for (uint32_t E : kBuckets) {
    if (ef_per_query) break;
    const uint32_t kk = std::min(k, E);
    if (dout.p) {
      cudaFree(dout.p);
      dout.p = nullptr;
    }
    cuda_ok(cudaMalloc(&dout.p, nq * kk * 16), "alloc");
    const double t_default = time_shape(E, kk, 0, 0, 0);
    double best = t_default;
    hgd_tune_entry pick{static_cast<uint32_t>(precision), E, 0, 0, 0, 0};
    const uint32_t c_full = std::max<uint32_t>(128, round_up32(E + 32));
    const uint32_t c_half = std::max<uint32_t>(128, round_up32(E / 2 + 32));
    for (uint32_t H : {512u, 1024u, 2048u, 4096u}) {
      if (H < 2 * E && H < 1024) continue;  // too small to hold a typical visited set
      for (uint32_t C : {c_full, c_half}) {
        if (C == c_half && c_half == c_full) continue;
        for (uint32_t wpb : {1u, 2u, 4u}) {
          if (static_cast<uint64_t>(wpb) * hgd_shape_smem_bytes(H, E, C) > kSmemPerBlock) continue;
          const double t = time_shape(E, kk, H, C, wpb);
          if (t < best) {
            best = t;
            pick.hash_slots = H;
            pick.cand_cap = C;
            pick.warps_per_block = wpb;
          }
        }
      }
    }
    table.push_back(pick);
    char buf[256];
    std::snprintf(buf, sizeof buf,
                  "%s    {\"precision\": %d, \"ef_hi\": %u, \"hash_slots\": %u, \"cand_cap\": %u, "
                  "\"warps_per_block\": %u, \"us_per_query\": %.4f, \"default_us_per_query\": %.4f}",
                  rows.empty() ? "" : ",\n", precision, E, pick.hash_slots, pick.cand_cap, pick.warps_per_block,
                  best, t_default);
    rows += buf;
    if (E >= ef_max) break;
  }
  const int rc = hgd_graph_set_tuning(g, table.data(), static_cast<uint32_t>(table.size()));
  if (rc != HGD_OK) throw std::runtime_error(std::string("autotune: ") + hgd_last_error());
  {
    std::lock_guard<std::mutex> dg(im.dev_mutex);
    im.tuning = table;
    im.launch_mode = launch_mode;
  }
  char name[256] = {0};
  uint32_t sms = 0;
  hgd_graph_device_info(g, name, sizeof name, &sms);
  char head[512];
  std::snprintf(head, sizeof head,
                "{\n  \"device\": \"%s\", \"sms\": %u, \"n\": %zu, \"dim\": %zu, \"M\": %zu, \"metric\": %d,\n"
                "  \"sample_queries\": %zu, \"k\": %u, \"launch_mode\": %d,\n  \"entries\": [\n",
                name, sms, im.count, im.dim, im.M, static_cast<int>(im.params.metric), nq, k, launch_mode);
  return std::string(head) + rows + "\n  ]\n}\n";
}

void apply_tuning_json(Index::Impl& im, const std::string& json) {
  // entries are flat objects with integer fields; read them in order
  auto field = [](const std::string& obj, const char* name, uint32_t* out) {
    const std::string key = std::string("\"") + name + "\"";
    const size_t p = obj.find(key);
    if (p == std::string::npos) return false;
    size_t c = obj.find(':', p + key.size());
    if (c == std::string::npos) return false;
    ++c;
    while (c < obj.size() && (obj[c] == ' ' || obj[c] == '\t' || obj[c] == '\n')) ++c;
    char* end = nullptr;
    const unsigned long v = std::strtoul(obj.c_str() + c, &end, 10);
    if (end == obj.c_str() + c) return false;
    *out = static_cast<uint32_t>(v);
    return true;
  };
  const size_t list = json.find("\"entries\"");
  if (list == std::string::npos) throw std::invalid_argument("tuning: no \"entries\" list");
  std::vector<hgd_tune_entry> table;
  size_t pos = json.find('[', list);
  const size_t stop = json.find(']', pos == std::string::npos ? list : pos);
  while (pos != std::string::npos) {
    const size_t a = json.find('{', pos);
    if (a == std::string::npos || a > stop) break;
    const size_t b = json.find('}', a);
    if (b == std::string::npos) throw std::invalid_argument("tuning: unterminated entry");
    const std::string obj = json.substr(a, b - a + 1);
    hgd_tune_entry e{};
    if (!field(obj, "precision", &e.precision) || !field(obj, "ef_hi", &e.ef_hi) ||
        !field(obj, "hash_slots", &e.hash_slots) || !field(obj, "cand_cap", &e.cand_cap) ||
        !field(obj, "warps_per_block", &e.warps_per_block))
      throw std::invalid_argument("tuning: entry without precision / ef_hi / hash_slots / cand_cap / warps_per_block");
    table.push_back(e);
    pos = b + 1;
  }
  uint32_t mode = static_cast<uint32_t>(im.launch_mode);
  const size_t mpos = json.find("\"launch_mode\"");
  if (mpos != std::string::npos && mpos < list) field(json.substr(mpos, 32), "launch_mode", &mode);
  if (mode > 1) throw std::invalid_argument("tuning: launch_mode must be 0 or 1");
  std::unique_lock<std::shared_mutex> lk(im.api_mutex);
  std::lock_guard<std::mutex> g(im.dev_mutex);
  if (im.dev && !table.empty()) {
    const int rc = hgd_graph_set_tuning(im.dev, table.data(), static_cast<uint32_t>(table.size()));
    if (rc != HGD_OK) throw std::invalid_argument(std::string("tuning: ") + hgd_last_error());
  }
  if (im.dev) hgd_graph_set_launch_mode(im.dev, static_cast<int>(mode));
  im.tuning = table;
  im.launch_mode = static_cast<int>(mode);
}

}  // namespace hnsw::gb
