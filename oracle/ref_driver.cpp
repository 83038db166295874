// ref_driver.cpp -- a small command-line driver that links the reference
// hnsw-engine library (compiled from its own sources by oracle/Makefile into
// oracle/_ref/) and exposes the calls the golden-fixture script needs:
// build + save with the reference's add_batch, load + search_batch, soft
// deletes, brute force and the raw distance kernels.  It is only built where
// the reference sources exist; nothing on the GPU path uses it.
//
// Raw file conventions: float32 / uint64 little-endian, row-major, no header.
// Result files hold nq*k records of {uint64 label, float32 distance}.

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>

#include "hnsw/filter.hpp"
#include "hnsw/index.hpp"
#include "hnsw/metric.hpp"

namespace {

template <typename T>
std::vector<T> read_raw(const std::string& path, std::size_t count) {
  std::vector<T> v(count);
  std::ifstream in(path, std::ios::binary);
  if (!in) throw std::runtime_error("cannot open " + path);
  if (count) in.read(reinterpret_cast<char*>(v.data()), static_cast<std::streamsize>(count * sizeof(T)));
  if (!in) throw std::runtime_error("short read " + path);
  return v;
}

void write_results(const std::string& path, const std::vector<hnsw::Neighbor>& out) {
  std::ofstream f(path, std::ios::binary | std::ios::trunc);
  for (const auto& nb : out) {
    f.write(reinterpret_cast<const char*>(&nb.label), 8);
    f.write(reinterpret_cast<const char*>(&nb.distance), 4);
  }
}

std::unique_ptr<hnsw::BitsetFilter> maybe_filter(int argc, char** argv, int at) {
  if (argc <= at + 1 || std::string(argv[at]) == "-") return nullptr;
  const uint64_t bits = std::stoull(argv[at + 1]);
  const auto words = read_raw<uint64_t>(argv[at], (bits + 63) / 64);
  auto f = std::make_unique<hnsw::BitsetFilter>(bits);
  for (uint64_t l = 0; l < bits; ++l)
    if ((words[l >> 6] >> (l & 63)) & 1ULL) f->set(l);
  return f;
}

int run(int argc, char** argv) {
  if (argc < 2) throw std::invalid_argument("usage: ref_driver <cmd> ...");
  const std::string cmd = argv[1];
  if (cmd == "isa") {
    std::cout << hnsw::simd::isa_name(hnsw::simd::active().isa) << "\n";
    return 0;
  }
  if (cmd == "build") {
    // build vecs n dim metric M efc seed threads out [labels]
    const std::size_t n = std::stoull(argv[3]), dim = std::stoull(argv[4]);
    hnsw::Params p;
    p.dim = dim;
    p.metric = hnsw::parse_metric(argv[5]);
    p.M = std::stoull(argv[6]);
    p.ef_construction = std::stoull(argv[7]);
    p.seed = std::stoull(argv[8]);
    const std::size_t threads = std::stoull(argv[9]);
    const auto vecs = read_raw<float>(argv[2], n * dim);
    std::vector<uint64_t> labels(n);
    if (argc > 11) labels = read_raw<uint64_t>(argv[11], n);
    else
      for (std::size_t i = 0; i < n; ++i) labels[i] = i;
    hnsw::Index index(p);
    if (n) index.add_batch(vecs.data(), labels.data(), n, threads);
    index.save(argv[10]);
    return 0;
  }
  if (cmd == "delete") {
    // delete in.idx labels.u64 count out.idx [set_ef]
    auto index = hnsw::Index::load(argv[2]);
    const std::size_t c = std::stoull(argv[4]);
    const auto labels = read_raw<uint64_t>(argv[3], c);
    for (auto l : labels) index.mark_deleted(l);
    if (argc > 6) index.set_ef(std::stoull(argv[6]));
    index.save(argv[5]);
    return 0;
  }
  if (cmd == "search") {
    // search idx queries nq k ef threads out [filter bits] ; mmap via env REF_MMAP=1
    const bool mm = std::getenv("REF_MMAP") && std::string(std::getenv("REF_MMAP")) == "1";
    auto index = hnsw::Index::load(argv[2], mm);
    const std::size_t nq = std::stoull(argv[4]), k = std::stoull(argv[5]), ef = std::stoull(argv[6]);
    const std::size_t threads = std::stoull(argv[7]);
    const auto qs = read_raw<float>(argv[3], nq * index.dim());
    auto f = maybe_filter(argc, argv, 9);
    std::vector<hnsw::Neighbor> out(nq * k);
    index.search_batch(qs.data(), nq, k, ef, out.data(), threads, f.get());
    write_results(argv[8], out);
    return 0;
  }
  if (cmd == "search1") {
    // search1 idx query k ef out [filter bits] -- Index::search (no padding)
    auto index = hnsw::Index::load(argv[2]);
    const std::size_t k = std::stoull(argv[4]), ef = std::stoull(argv[5]);
    const auto q = read_raw<float>(argv[3], index.dim());
    auto f = maybe_filter(argc, argv, 7);
    const auto res = index.search(q.data(), k, ef, f.get());
    write_results(argv[6], res);
    return 0;
  }
  if (cmd == "bf") {
    // bf vecs n dim metric queries nq k threads out [filter bits]
    const std::size_t n = std::stoull(argv[3]), dim = std::stoull(argv[4]);
    const auto metric = hnsw::parse_metric(argv[5]);
    const std::size_t nq = std::stoull(argv[7]), k = std::stoull(argv[8]), threads = std::stoull(argv[9]);
    const auto vecs = read_raw<float>(argv[2], n * dim);
    const auto qs = read_raw<float>(argv[6], nq * dim);
    auto f = maybe_filter(argc, argv, 11);
    hnsw::BruteForceIndex bf(dim, metric);
    bf.add(vecs.data(), nullptr, n);
    std::vector<hnsw::Neighbor> out(nq * k);
    bf.search_batch(qs.data(), nq, k, out.data(), threads, f.get());
    write_results(argv[10], out);
    return 0;
  }
  if (cmd == "kernel") {
    // kernel isa a b dim out: writes {l2, dot} float32 for each of count pairs
    const auto isa = hnsw::simd::parse_isa(argv[2]);
    const std::size_t dim = std::stoull(argv[5]), count = std::stoull(argv[6]);
    const auto a = read_raw<float>(argv[3], dim * count);
    const auto b = read_raw<float>(argv[4], dim * count);
    const auto& k = hnsw::simd::get(isa);
    std::ofstream f(argv[7], std::ios::binary | std::ios::trunc);
    for (std::size_t i = 0; i < count; ++i) {
      const float l2 = k.l2_sq(a.data() + i * dim, b.data() + i * dim, dim);
      const float dp = k.dot(a.data() + i * dim, b.data() + i * dim, dim);
      f.write(reinterpret_cast<const char*>(&l2), 4);
      f.write(reinterpret_cast<const char*>(&dp), 4);
    }
    return 0;
  }
  if (cmd == "load") {
    // load idx [mmap]: exit 0 if it loads, 3 if it throws runtime_error
    try {
      auto index = hnsw::Index::load(argv[2], argc > 3 && std::string(argv[3]) == "1");
      std::cout << "ok " << index.size() << "\n";
      return 0;
    } catch (const std::runtime_error& e) {
      std::cout << "error " << e.what() << "\n";
      return 3;
    }
  }
  throw std::invalid_argument("unknown command " + cmd);
}

}  // namespace

int main(int argc, char** argv) {
  try {
    return run(argc, argv);
  } catch (const std::exception& e) {
    std::cerr << "ref_driver: " << e.what() << "\n";
    return 2;
  }
}
