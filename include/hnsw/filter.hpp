#pragma once
// Label filters, declared as in the reference's include/hnsw/filter.hpp:1-50.
// On the GPU a filter becomes a bitset over internal ids: a BitsetFilter is
// translated with one pass over the index's labels, any other Filter is
// evaluated once per node on the host (it must be a pure function of the
// label, as the reference's thread-safety contract already requires).

#include <cstdint>
#include <functional>
#include <vector>

namespace hnsw {

class Filter {
 public:
  virtual ~Filter() = default;
  virtual bool allowed(uint64_t label) const = 0;
  bool operator()(uint64_t label) const { return allowed(label); }
};

class FunctionFilter final : public Filter {
 public:
  explicit FunctionFilter(std::function<bool(uint64_t)> fn);
  bool allowed(uint64_t label) const override { return fn_(label); }

 private:
  std::function<bool(uint64_t)> fn_;
};

/// Allow-list stored as a bitset indexed by label. Labels >= size() are rejected.
class BitsetFilter final : public Filter {
 public:
  BitsetFilter() = default;
  explicit BitsetFilter(uint64_t num_labels);
  static BitsetFilter from_labels(const uint64_t* labels, std::size_t n);

  void set(uint64_t label, bool value = true);
  bool allowed(uint64_t label) const override {
    return label < size_ && ((words_[label >> 6] >> (label & 63)) & 1ULL) != 0;
  }
  uint64_t size() const noexcept { return size_; }
  std::size_t count() const noexcept;
  /// Raw words (bit l of word l/64), for the device translation.
  const uint64_t* words() const noexcept { return words_.data(); }

 private:
  std::vector<uint64_t> words_;
  uint64_t size_ = 0;
};

}  // namespace hnsw
