// bruteforce.cpp -- hnsw::BruteForceIndex (reference src/brute_force.cpp:20-69)
// answered on the GPU by the exact k-NN kernels behind hgd_flat / hgd_bruteforce.
#include <cmath>
#include <limits>
#include <stdexcept>
#include <string>

#include "graph.hpp"

namespace hnsw {

struct BruteForceIndex::Dev {
  hgd_flat* flat = nullptr;
  std::size_t rows = 0;  // rows uploaded
  ~Dev() {
    if (flat) hgd_flat_free(flat);
  }
};

namespace {
void prepare_row(Metric m, const float* src, float* dst, std::size_t dim) {
  if (m != Metric::Cosine) {
    for (std::size_t i = 0; i < dim; ++i) dst[i] = src[i];
    return;
  }
  double norm = 0.0;
  for (std::size_t i = 0; i < dim; ++i) norm += static_cast<double>(src[i]) * src[i];
  const float inv = norm > 0.0 ? static_cast<float>(1.0 / std::sqrt(norm)) : 1.0f;
  for (std::size_t i = 0; i < dim; ++i) dst[i] = src[i] * inv;
}
}  // namespace

BruteForceIndex::BruteForceIndex(std::size_t dim, Metric metric) : dim_(dim), metric_(metric) {
  if (dim == 0) throw std::invalid_argument("BruteForceIndex: dim must be > 0");
}
BruteForceIndex::~BruteForceIndex() = default;
BruteForceIndex::BruteForceIndex(BruteForceIndex&&) noexcept = default;
BruteForceIndex& BruteForceIndex::operator=(BruteForceIndex&&) noexcept = default;

void BruteForceIndex::add(const float* vecs, const uint64_t* labels, std::size_t n) {
  const std::size_t old = labels_.size();
  data_.resize((old + n) * dim_);
  labels_.resize(old + n);
  for (std::size_t i = 0; i < n; ++i) {
    prepare_row(metric_, vecs + i * dim_, data_.data() + (old + i) * dim_, dim_);
    labels_[old + i] = labels != nullptr ? labels[i] : static_cast<uint64_t>(old + i);
  }
  dev_.reset();
}

void BruteForceIndex::search_batch(const float* qs, std::size_t nq, std::size_t k, Neighbor* out,
                                   std::size_t /*num_threads*/, const Filter* f) const {
  if (k == 0) throw std::invalid_argument("search: k must be > 0");
  if (nq == 0) return;
  if (qs == nullptr || out == nullptr) throw std::invalid_argument("search_batch: null pointer");
  if (labels_.empty()) {
    for (std::size_t i = 0; i < nq * k; ++i) out[i] = Neighbor{kInvalidLabel, std::numeric_limits<float>::infinity()};
    return;
  }
  if (!dev_) {
    auto d = std::make_unique<Dev>();
    const int rc = hgd_flat_upload(data_.data(), labels_.data(), labels_.size(), dim_, static_cast<int>(metric_), 0,
                                   static_cast<int>(simd::active().isa), &d->flat);
    if (rc != HGD_OK) {
      const std::string msg = std::string("BruteForceIndex upload: ") + hgd_last_error();
      if (rc == HGD_EINVAL) throw std::invalid_argument(msg);
      throw std::runtime_error(msg);
    }
    d->rows = labels_.size();
    dev_ = std::move(d);
  }
  std::vector<uint64_t> words;
  hgd_bitset view{};
  if (f != nullptr) {
    // label-space bitset over the labels present
    uint64_t top = 0;
    for (uint64_t l : labels_) top = l > top ? l : top;
    if (const auto* bs = dynamic_cast<const BitsetFilter*>(f)) {
      view.words = bs->words();
      view.num_bits = bs->size();
    } else {
      // arbitrary predicate: evaluate per row, pass an id-space bitset
      words.assign((labels_.size() + 63) / 64, 0);
      for (std::size_t i = 0; i < labels_.size(); ++i)
        if (f->allowed(labels_[i])) words[i >> 6] |= 1ULL << (i & 63);
      view.words = words.data();
      view.num_bits = labels_.size();
      view.label_space = 0;
    }
    if (view.words == nullptr && view.num_bits == 0) view.label_space = 1;
    if (dynamic_cast<const BitsetFilter*>(f)) view.label_space = 1;
  }
  hgd_flat_set_path(dev_->flat, path_);
  const int rc = hgd_bruteforce(dev_->flat, qs, nq, static_cast<uint32_t>(k), f ? &view : nullptr, out, nullptr);
  last_path_ = hgd_flat_last_path(dev_->flat);
  if (rc != HGD_OK) {
    const std::string msg = std::string("BruteForceIndex search: ") + hgd_last_error();
    if (rc == HGD_EINVAL) throw std::invalid_argument(msg);
    throw std::runtime_error(msg);
  }
}

void BruteForceIndex::set_gpu_path(int path) {
  if (path < 0 || path > 2) throw std::invalid_argument("set_gpu_path: 0 (auto), 1 (scan) or 2 (tensor)");
  path_ = path;
}

std::vector<Neighbor> BruteForceIndex::search(const float* q, std::size_t k, const Filter* f) const {
  if (k == 0) throw std::invalid_argument("search: k must be > 0");
  std::vector<Neighbor> row(k);
  search_batch(q, 1, k, row.data(), 0, f);
  std::size_t m = 0;
  while (m < k && row[m].label != kInvalidLabel) ++m;
  row.resize(m);
  return row;
}

}  // namespace hnsw
