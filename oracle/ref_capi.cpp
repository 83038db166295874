// ref_capi.cpp -- a C shim over the reference hnsw-engine library, compiled
// with the reference's own sources (oracle/Makefile) into
// oracle/_ref/libhnswref.so.  Test and benchmark infrastructure only: it
// lets Python build graphs with the reference's add_batch
// (src/index.cpp:273-306), load them (src/persist.cpp:476-541) and time the
// reference's own search_batch (src/search_layer.cpp:180-194) and brute
// force (src/brute_force.cpp:34-69) in process, through ctypes.  Nothing on
// the GPU path links it.
//
// Every entry returns 0 on success, or -1 with the exception's message
// copied into the caller's err buffer.

#include <cstdint>
#include <cstring>
#include <exception>
#include <memory>
#include <string>
#include <vector>

#include "hnsw/filter.hpp"
#include "hnsw/index.hpp"
#include "hnsw/metric.hpp"

#define REF_API extern "C" __attribute__((visibility("default")))

namespace {

int fail(const std::exception& e, char* err, std::size_t errn) {
  if (err && errn) {
    std::strncpy(err, e.what(), errn - 1);
    err[errn - 1] = '\0';
  }
  return -1;
}

template <typename F>
int guarded(char* err, std::size_t errn, F&& f) {
  try {
    f();
    return 0;
  } catch (const std::exception& e) {
    return fail(e, err, errn);
  }
}

std::vector<uint64_t> iota_labels(std::size_t n) {
  std::vector<uint64_t> v(n);
  for (std::size_t i = 0; i < n; ++i) v[i] = i;
  return v;
}

}  // namespace

// name of the distance kernel the reference dispatched to on this host
REF_API int ref_isa(char* out, std::size_t n) {
  const std::string s(hnsw::simd::isa_name(hnsw::simd::active().isa));
  if (n == 0) return -1;
  std::strncpy(out, s.c_str(), n - 1);
  out[n - 1] = '\0';
  return 0;
}

// add_batch over n rows (labels 0..n-1 when labels is null) and save
REF_API int ref_build(const float* vecs, const uint64_t* labels, std::size_t n, std::size_t dim, const char* metric,
                      std::size_t M, std::size_t efc, uint64_t seed, std::size_t threads, const char* path, char* err,
                      std::size_t errn) {
  return guarded(err, errn, [&] {
    hnsw::Params p;
    p.dim = dim;
    p.metric = hnsw::parse_metric(metric);
    p.M = M;
    p.ef_construction = efc;
    p.seed = seed;
    std::vector<uint64_t> own;
    if (!labels) {
      own = iota_labels(n);
      labels = own.data();
    }
    hnsw::Index index(p);
    if (n) index.add_batch(vecs, labels, n, threads);
    index.save(path);
  });
}

REF_API int ref_load(const char* path, int mmap, void** out, char* err, std::size_t errn) {
  return guarded(err, errn, [&] { *out = new hnsw::Index(hnsw::Index::load(path, mmap != 0)); });
}

REF_API void ref_free(void* ix) { delete static_cast<hnsw::Index*>(ix); }

REF_API int ref_info(void* ix, uint64_t* out4) {
  const auto* x = static_cast<const hnsw::Index*>(ix);
  out4[0] = x->size();
  out4[1] = x->dim();
  out4[2] = x->ef();
  out4[3] = static_cast<uint64_t>(x->max_level());
  return 0;
}

REF_API int ref_mark_deleted(void* ix, uint64_t label, char* err, std::size_t errn) {
  return guarded(err, errn, [&] { static_cast<hnsw::Index*>(ix)->mark_deleted(label); });
}

REF_API int ref_set_ef(void* ix, std::size_t ef, char* err, std::size_t errn) {
  return guarded(err, errn, [&] { static_cast<hnsw::Index*>(ix)->set_ef(ef); });
}

REF_API int ref_save(void* ix, const char* path, char* err, std::size_t errn) {
  return guarded(err, errn, [&] { static_cast<const hnsw::Index*>(ix)->save(path); });
}

// a BitsetFilter over label space [0, bits) from little-endian words
REF_API void* ref_filter_new(const uint64_t* words, uint64_t bits) {
  auto* f = new hnsw::BitsetFilter(bits);
  for (uint64_t w = 0; w < (bits + 63) / 64; ++w) {
    uint64_t x = words[w];
    while (x) {
      const int b = __builtin_ctzll(x);
      x &= x - 1;
      f->set(w * 64 + static_cast<uint64_t>(b));
    }
  }
  return f;
}

REF_API void ref_filter_free(void* f) { delete static_cast<hnsw::BitsetFilter*>(f); }

// Index::search_batch: out holds nq * k Neighbor records {u64 label, f32 dist, 4 B pad}
REF_API int ref_search_batch(void* ix, const float* qs, std::size_t nq, std::size_t k, std::size_t ef, void* out,
                             std::size_t threads, const void* filter, char* err, std::size_t errn) {
  return guarded(err, errn, [&] {
    static_cast<const hnsw::Index*>(ix)->search_batch(qs, nq, k, ef, static_cast<hnsw::Neighbor*>(out), threads,
                                                      static_cast<const hnsw::Filter*>(filter));
  });
}

// Index::search (one query, no padding); *count receives the result size
REF_API int ref_search(void* ix, const float* q, std::size_t k, std::size_t ef, const void* filter, void* out,
                       std::size_t* count, char* err, std::size_t errn) {
  return guarded(err, errn, [&] {
    const auto r = static_cast<const hnsw::Index*>(ix)->search(q, k, ef, static_cast<const hnsw::Filter*>(filter));
    std::memcpy(out, r.data(), r.size() * sizeof(hnsw::Neighbor));
    *count = r.size();
  });
}

// BruteForceIndex::search_batch over n rows (labels 0..n-1 when null)
REF_API int ref_bruteforce(const float* vecs, const uint64_t* labels, std::size_t n, std::size_t dim,
                           const char* metric, const float* qs, std::size_t nq, std::size_t k, void* out,
                           std::size_t threads, const void* filter, char* err, std::size_t errn) {
  return guarded(err, errn, [&] {
    hnsw::BruteForceIndex bf(dim, hnsw::parse_metric(metric));
    std::vector<uint64_t> own;
    if (!labels) {
      own = iota_labels(n);
      labels = own.data();
    }
    bf.add(vecs, labels, n);
    bf.search_batch(qs, nq, k, static_cast<hnsw::Neighbor*>(out), threads, static_cast<const hnsw::Filter*>(filter));
  });
}

// raw kernel values of the named ISA's table over count row pairs
// (out[2i] = l2_sq, out[2i+1] = dot); -1 if the ISA is not available here
REF_API int ref_kernels(const char* isa, const float* a, const float* b, std::size_t dim, std::size_t count,
                        float* out, char* err, std::size_t errn) {
  return guarded(err, errn, [&] {
    const auto& k = hnsw::simd::get(hnsw::simd::parse_isa(isa));
    for (std::size_t i = 0; i < count; ++i) {
      out[2 * i] = k.l2_sq(a + i * dim, b + i * dim, dim);
      out[2 * i + 1] = k.dot(a + i * dim, b + i * dim, dim);
    }
  });
}
