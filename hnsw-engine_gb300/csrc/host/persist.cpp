// persist.cpp -- FORMAT v1 (the reference's on-disk index, docs/FORMAT.md):
// a 256-byte header, then six 64-byte aligned sections (vectors, level0,
// labels, levels, deleted, upper) separated by zero padding.
//
// Reading follows the reference's validation order (src/persist.cpp:245-365,
// 476-541): header size, magic, endianness, version, header FNV-1a, file
// size, scalar ranges, section offsets, zero padding, payload hash, then the
// graph itself.  Any failure throws std::runtime_error("corrupt or
// incompatible index file '<path>': <reason>").  Writing produces the same
// bytes as the reference's Index::save for the same state.
#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <cstring>
#include <fstream>
#include <shared_mutex>
#include <stdexcept>
#include <string>

#include "graph.hpp"

namespace hnsw {
namespace gb {

Mapping::Mapping(const std::string& path) {
  const int fd = ::open(path.c_str(), O_RDONLY);
  if (fd < 0) throw std::runtime_error("cannot open " + path);
  struct stat st {};
  if (::fstat(fd, &st) != 0) {
    ::close(fd);
    throw std::runtime_error("cannot stat " + path);
  }
  if (st.st_size <= 0) {
    ::close(fd);
    throw std::runtime_error(path + ": empty file");
  }
  void* p = ::mmap(nullptr, static_cast<std::size_t>(st.st_size), PROT_READ, MAP_PRIVATE, fd, 0);
  ::close(fd);
  if (p == MAP_FAILED) throw std::runtime_error("mmap failed for " + path);
  data_ = static_cast<const unsigned char*>(p);
  size_ = static_cast<std::size_t>(st.st_size);
}
Mapping::~Mapping() { reset(); }
Mapping::Mapping(Mapping&& o) noexcept : data_(o.data_), size_(o.size_) {
  o.data_ = nullptr;
  o.size_ = 0;
}
Mapping& Mapping::operator=(Mapping&& o) noexcept {
  if (this != &o) {
    reset();
    data_ = o.data_;
    size_ = o.size_;
    o.data_ = nullptr;
    o.size_ = 0;
  }
  return *this;
}
void Mapping::reset() noexcept {
  if (data_) ::munmap(const_cast<unsigned char*>(data_), size_);
  data_ = nullptr;
  size_ = 0;
}

}  // namespace gb

namespace {

constexpr std::size_t kHeaderBytes = 256;
constexpr std::size_t kSectionAlign = 64;
constexpr char kMagic[8] = {'H', 'N', 'S', 'W', 'E', 'N', 'G', '\0'};
constexpr uint32_t kFormatVersion = 1;
constexpr uint32_t kEndianMark = 0x01020304;

// header field byte offsets (FORMAT.md header table)
enum HeaderAt : std::size_t {
  kAtMagic = 0, kAtVersion = 8, kAtEndian = 12, kAtDim = 16, kAtMetric = 24, kAtM = 32, kAtEfc = 40,
  kAtEfSearch = 48, kAtSeed = 56, kAtMaxElems = 64, kAtCount = 72, kAtPaddedDim = 80, kAtMaxLevel = 88,
  kAtEntry = 92, kAtUpperUsed = 96, kAtNumDeleted = 104, kAtRng = 112, kAtOffVec = 120, kAtOffL0 = 128,
  kAtOffLabels = 136, kAtOffLevels = 144, kAtOffDeleted = 152, kAtOffUpper = 160, kAtFileSize = 168,
  kAtPayload = 176, kAtHeaderSum = 184
};

template <typename T>
T peek(const unsigned char* b, std::size_t at) {
  T v;
  std::memcpy(&v, b + at, sizeof v);
  return v;
}
template <typename T>
void poke(unsigned char* b, std::size_t at, T v) {
  std::memcpy(b + at, &v, sizeof v);
}

uint64_t fnv1a64(const unsigned char* p, std::size_t n) noexcept {
  uint64_t h = 0xcbf29ce484222325ULL;
  for (std::size_t i = 0; i < n; ++i) h = (h ^ p[i]) * 0x100000001b3ULL;
  return h;
}

uint64_t header_sum(const unsigned char* hdr) noexcept {
  unsigned char copy[kHeaderBytes];
  std::memcpy(copy, hdr, kHeaderBytes);
  std::memset(copy + kAtHeaderSum, 0, 8);
  return fnv1a64(copy, kHeaderBytes);
}

/// FORMAT v1 payload hash (FORMAT.md "Payload checksum").
class SectionHash {
 public:
  // one whole section
  void feed(const void* data, std::size_t n) noexcept { feed_part(data, n, true, n); }
  // a section in consecutive parts: every part but the last a multiple of 8
  // bytes long; `last` closes the section of `total` bytes (the same value
  // as one feed of the whole section)
  void feed_part(const void* data, std::size_t n, bool last, std::size_t total) noexcept {
    const auto* p = static_cast<const unsigned char*>(data);
    std::size_t i = 0;
    for (; i + 8 <= n; i += 8) {
      uint64_t w;
      std::memcpy(&w, p + i, 8);
      step(w);
    }
    if (!last) return;
    for (; i < n; ++i) step(0x100ULL | p[i]);
    step(total);
  }
  uint64_t value() const noexcept { return h_; }

 private:
  void step(uint64_t w) noexcept {
    h_ ^= w * 0x9E3779B97F4A7C15ULL;
    h_ = (h_ << 31) | (h_ >> 33);
    h_ *= 0xC2B2AE3D27D4EB4FULL;
  }
  uint64_t h_ = 0x243F6A8885A308D3ULL;
};

struct Fields {
  uint64_t dim = 0, M = 0, efc = 0, ef_search = 0, seed = 0, max_elements = 0, count = 0, padded_dim = 0;
  uint32_t metric = 0, entry = gb::kNoNode;
  int32_t max_level = -1;
  uint64_t upper_used = 0, num_deleted = 0, rng = 0;
  uint64_t off[6] = {};  // vectors, level0, labels, levels, deleted, upper
  uint64_t file_size = 0, payload = 0;
};

struct Sizes {
  std::size_t bytes[6];
};

Sizes section_bytes(uint64_t count, uint64_t pd, uint64_t M, uint64_t upper_used) {
  return Sizes{{count * pd * 4, count * (1 + 2 * M) * 4, count * 8, count, count, upper_used * 4}};
}

uint64_t align64(uint64_t v) { return (v + kSectionAlign - 1) / kSectionAlign * kSectionAlign; }

void layout(Fields& f) {
  const Sizes s = section_bytes(f.count, f.padded_dim, f.M, f.upper_used);
  uint64_t pos = kHeaderBytes;
  for (int i = 0; i < 6; ++i) {
    f.off[i] = pos;
    pos = i < 5 ? align64(pos + s.bytes[i]) : pos + s.bytes[i];
  }
  f.file_size = pos;
}

[[noreturn]] void corrupt(const std::string& path, const std::string& why) {
  throw std::runtime_error("corrupt or incompatible index file '" + path + "': " + why);
}

Fields parse_header(const unsigned char* b, std::size_t actual, const std::string& path) {
  if (actual < kHeaderBytes) corrupt(path, "file too small for header");
  if (std::memcmp(b + kAtMagic, kMagic, 8) != 0) corrupt(path, "bad magic");
  if (peek<uint32_t>(b, kAtEndian) != kEndianMark) corrupt(path, "endianness mismatch");
  if (peek<uint32_t>(b, kAtVersion) != kFormatVersion)
    corrupt(path, "unsupported version " + std::to_string(peek<uint32_t>(b, kAtVersion)));
  if (peek<uint64_t>(b, kAtHeaderSum) != header_sum(b)) corrupt(path, "header checksum mismatch");
  Fields f;
  f.dim = peek<uint64_t>(b, kAtDim);
  f.metric = peek<uint32_t>(b, kAtMetric);
  f.M = peek<uint64_t>(b, kAtM);
  f.efc = peek<uint64_t>(b, kAtEfc);
  f.ef_search = peek<uint64_t>(b, kAtEfSearch);
  f.seed = peek<uint64_t>(b, kAtSeed);
  f.max_elements = peek<uint64_t>(b, kAtMaxElems);
  f.count = peek<uint64_t>(b, kAtCount);
  f.padded_dim = peek<uint64_t>(b, kAtPaddedDim);
  f.max_level = peek<int32_t>(b, kAtMaxLevel);
  f.entry = peek<uint32_t>(b, kAtEntry);
  f.upper_used = peek<uint64_t>(b, kAtUpperUsed);
  f.num_deleted = peek<uint64_t>(b, kAtNumDeleted);
  f.rng = peek<uint64_t>(b, kAtRng);
  for (int i = 0; i < 6; ++i) f.off[i] = peek<uint64_t>(b, kAtOffVec + 8 * static_cast<std::size_t>(i));
  f.file_size = peek<uint64_t>(b, kAtFileSize);
  f.payload = peek<uint64_t>(b, kAtPayload);

  if (f.file_size != actual) corrupt(path, "size mismatch (truncated or extended file)");
  if (f.dim == 0 || f.dim > (1u << 20)) corrupt(path, "invalid dim");
  if (f.metric > 2) corrupt(path, "invalid metric");
  if (f.M < 2 || f.M > 2048) corrupt(path, "invalid M");
  if (f.efc == 0 || f.ef_search == 0) corrupt(path, "invalid ef");
  if (f.padded_dim != gb::round_up(f.dim, gb::kPadFloats)) corrupt(path, "invalid padded dim");
  if (f.count > actual || f.count >= gb::kNoNode) corrupt(path, "invalid count");
  if (f.upper_used > actual) corrupt(path, "invalid upper size");
  if (f.num_deleted > f.count) corrupt(path, "invalid deleted count");
  if (f.max_elements != 0 && (f.max_elements < f.count || f.max_elements >= gb::kNoNode))
    corrupt(path, "invalid max_elements");
  if (f.count == 0) {
    if (f.max_level != -1 || f.entry != gb::kNoNode) corrupt(path, "invalid empty-index header");
  } else if (f.max_level < 0 || f.max_level > gb::kMaxLevel || f.entry >= f.count) {
    corrupt(path, "invalid entry point / max level");
  }
  Fields want = f;
  layout(want);
  for (int i = 0; i < 6; ++i)
    if (want.off[i] != f.off[i]) corrupt(path, "section offsets inconsistent with header");
  if (want.file_size != f.file_size) corrupt(path, "section offsets inconsistent with header");
  return f;
}

Params params_of(const Fields& f) {
  Params p;
  p.dim = f.dim;
  p.metric = static_cast<Metric>(f.metric);
  p.M = f.M;
  p.ef_construction = f.efc;
  p.max_elements = 0;
  p.seed = f.seed;
  return p;
}

/// The state of a read-only index whose arrays stay in the file mapping b.
void bind_mapped(Index::Impl& im, const Fields& f, const unsigned char* b) {
  im.params.max_elements = f.max_elements;
  im.count = im.capacity = f.count;
  im.ef_search = f.ef_search;
  im.upper_used = f.upper_used;
  im.entry_point = f.entry;
  im.max_level = f.max_level;
  im.rng_state = f.rng;
  im.vecs = reinterpret_cast<const float*>(b + f.off[0]);
  im.l0 = const_cast<uint32_t*>(reinterpret_cast<const uint32_t*>(b + f.off[1]));
  im.labels = reinterpret_cast<const uint64_t*>(b + f.off[2]);
  im.levels = b + f.off[3];
  im.upper = const_cast<uint32_t*>(reinterpret_cast<const uint32_t*>(b + f.off[5]));
}

/// pread until `n` bytes are in or the file ends; false on a short read.
bool pread_full(int fd, void* dst, uint64_t n, uint64_t at) {
  auto* p = static_cast<unsigned char*>(dst);
  while (n > 0) {
    const ssize_t r = ::pread(fd, p, static_cast<std::size_t>(std::min<uint64_t>(n, 1ull << 30)), static_cast<off_t>(at));
    if (r <= 0) return false;
    p += r;
    at += static_cast<uint64_t>(r);
    n -= static_cast<uint64_t>(r);
  }
  return true;
}

/// Graph checks and derived state (reference persist.cpp:321-365).
void check_graph(Index::Impl& im, const Fields& f, const uint8_t* tomb, const std::string& path) {
  const std::size_t n = f.count;
  im.upper_offset.assign(n, 0);
  uint64_t pos = 0;
  for (std::size_t i = 0; i < n; ++i) {
    if (im.levels[i] > f.max_level) corrupt(path, "node level exceeds max level");
    im.upper_offset[i] = pos;
    pos += static_cast<uint64_t>(im.levels[i]) * im.upper_stride;
  }
  if (pos != f.upper_used) corrupt(path, "upper-layer size does not match levels");
  if (n > 0 && im.levels[f.entry] != f.max_level) corrupt(path, "entry point is not on the top level");
  for (std::size_t i = 0; i < n; ++i) {
    for (int lc = 0; lc <= im.levels[i]; ++lc) {
      const uint32_t* l = im.list(static_cast<uint32_t>(i), lc);
      if (l[0] > im.degree_cap(lc)) corrupt(path, "neighbor count exceeds maximum degree");
      for (uint32_t j = 1; j <= l[0]; ++j)
        if (l[j] >= n || im.levels[l[j]] < lc) corrupt(path, "neighbor id out of range");
    }
  }
  im.label_to_id.clear();
  im.label_to_id.reserve(n);
  for (std::size_t i = 0; i < n; ++i)
    if (!im.label_to_id.emplace(im.labels[i], static_cast<uint32_t>(i)).second) corrupt(path, "duplicate label");
  im.deleted.assign(tomb, tomb + n);
  std::size_t dels = 0;
  for (uint8_t d : im.deleted) {
    if (d > 1) corrupt(path, "invalid tombstone byte");
    dels += d;
  }
  if (dels != f.num_deleted) corrupt(path, "deleted count mismatch");
  im.num_deleted = dels;
}

}  // namespace

void Index::save(const std::string& path) const {
  std::shared_lock<std::shared_mutex> lk(impl_->api_mutex);
  const Impl& im = *impl_;
  Fields f;
  f.dim = im.dim;
  f.metric = static_cast<uint32_t>(im.params.metric);
  f.M = im.M;
  f.efc = im.params.ef_construction;
  f.ef_search = im.ef_search;
  f.seed = im.params.seed;
  f.max_elements = im.params.max_elements;
  f.count = im.count;
  f.padded_dim = im.padded_dim;
  f.max_level = im.max_level;
  f.entry = im.entry_point;
  f.upper_used = im.upper_used;
  f.num_deleted = im.num_deleted;
  f.rng = im.rng_state;
  layout(f);
  const Sizes s = section_bytes(f.count, f.padded_dim, f.M, f.upper_used);
  const void* src[6] = {im.vecs, im.l0, im.labels, im.levels, im.deleted.data(), im.upper};
  SectionHash hash;
  for (int i = 0; i < 6; ++i) hash.feed(src[i], s.bytes[i]);
  f.payload = hash.value();

  unsigned char hdr[kHeaderBytes] = {};
  std::memcpy(hdr + kAtMagic, kMagic, 8);
  poke<uint32_t>(hdr, kAtVersion, kFormatVersion);
  poke<uint32_t>(hdr, kAtEndian, kEndianMark);
  poke(hdr, kAtDim, f.dim);
  poke(hdr, kAtMetric, f.metric);
  poke(hdr, kAtM, f.M);
  poke(hdr, kAtEfc, f.efc);
  poke(hdr, kAtEfSearch, f.ef_search);
  poke(hdr, kAtSeed, f.seed);
  poke(hdr, kAtMaxElems, f.max_elements);
  poke(hdr, kAtCount, f.count);
  poke(hdr, kAtPaddedDim, f.padded_dim);
  poke(hdr, kAtMaxLevel, f.max_level);
  poke(hdr, kAtEntry, f.entry);
  poke(hdr, kAtUpperUsed, f.upper_used);
  poke(hdr, kAtNumDeleted, f.num_deleted);
  poke(hdr, kAtRng, f.rng);
  for (int i = 0; i < 6; ++i) poke(hdr, kAtOffVec + 8 * static_cast<std::size_t>(i), f.off[i]);
  poke(hdr, kAtFileSize, f.file_size);
  poke(hdr, kAtPayload, f.payload);
  poke(hdr, kAtHeaderSum, header_sum(hdr));

  std::ofstream out(path, std::ios::binary | std::ios::trunc);
  if (!out) throw std::runtime_error("cannot open " + path + " for writing");
  out.write(reinterpret_cast<const char*>(hdr), kHeaderBytes);
  static const char zeros[kSectionAlign] = {};
  uint64_t pos = kHeaderBytes;
  for (int i = 0; i < 6; ++i) {
    out.write(zeros, static_cast<std::streamsize>(f.off[i] - pos));
    if (s.bytes[i]) out.write(static_cast<const char*>(src[i]), static_cast<std::streamsize>(s.bytes[i]));
    pos = f.off[i] + s.bytes[i];
  }
  out.flush();
  if (!out) throw std::runtime_error("write failed: " + path);
}

Index Index::load(const std::string& path, bool mmap) {
  if (mmap) {
    gb::Mapping file(path);
    const unsigned char* b = file.data();
    const Fields f = parse_header(b, file.size(), path);
    auto im = std::make_unique<Impl>(params_of(f));
    bind_mapped(*im, f, b);
    const Sizes s = section_bytes(f.count, f.padded_dim, f.M, f.upper_used);
    SectionHash hash;
    uint64_t pos = kHeaderBytes;
    for (int i = 0; i < 6; ++i) {
      for (uint64_t p = pos; p < f.off[i]; ++p)
        if (b[p] != 0) corrupt(path, "non-zero padding");
      hash.feed(b + f.off[i], s.bytes[i]);
      pos = f.off[i] + s.bytes[i];
    }
    if (hash.value() != f.payload) corrupt(path, "payload checksum mismatch");
    check_graph(*im, f, b + f.off[4], path);
    im->mapping = std::move(file);
    im->read_only = true;
    return Index(std::move(im));
  }

  std::ifstream in(path, std::ios::binary | std::ios::ate);
  if (!in) throw std::runtime_error("cannot open " + path);
  const auto actual = static_cast<std::size_t>(in.tellg());
  if (actual < kHeaderBytes) corrupt(path, "file too small for header");
  unsigned char hdr[kHeaderBytes];
  in.seekg(0);
  if (!in.read(reinterpret_cast<char*>(hdr), kHeaderBytes)) corrupt(path, "short read");
  const Fields f = parse_header(hdr, actual, path);
  auto im = std::make_unique<Impl>(params_of(f));
  im->params.max_elements = f.max_elements;
  if (f.count > 0) im->grow(std::max<std::size_t>(f.count, f.max_elements));
  const Sizes s = section_bytes(f.count, f.padded_dim, f.M, f.upper_used);
  std::vector<uint8_t> tomb(f.count);
  im->upper_store.assign(f.upper_used, 0u);
  void* dst[6] = {im->vec_store.data(), im->l0_store.data(), im->label_store.data(), im->level_store.data(),
                  tomb.data(), im->upper_store.data()};
  SectionHash hash;
  uint64_t pos = kHeaderBytes;
  for (int i = 0; i < 6; ++i) {
    char pad[kSectionAlign];
    const uint64_t gap = f.off[i] - pos;
    if (gap > sizeof pad || (gap && !in.read(pad, static_cast<std::streamsize>(gap)))) corrupt(path, "short read");
    for (uint64_t p = 0; p < gap; ++p)
      if (pad[p] != 0) corrupt(path, "non-zero padding");
    if (s.bytes[i] && !in.read(static_cast<char*>(dst[i]), static_cast<std::streamsize>(s.bytes[i])))
      corrupt(path, "short read");
    hash.feed(dst[i], s.bytes[i]);
    pos = f.off[i] + s.bytes[i];
  }
  if (hash.value() != f.payload) corrupt(path, "payload checksum mismatch");
  im->bind_pointers();
  im->count = f.count;
  im->ef_search = f.ef_search;
  im->upper_used = f.upper_used;
  im->entry_point = f.entry;
  im->max_level = f.max_level;
  im->rng_state = f.rng;
  check_graph(*im, f, tomb.data(), path);
  im->deleted.resize(im->capacity, 0);
  return Index(std::move(im));
}

Index Index::load_to_device(const std::string& path, int device, bool mmap) {
  // The checks and their order are load()'s; the reads go through the
  // stream's pinned buffers for sections 0-2 (hashed there, copied to the
  // host arrays unless mapped, and sent to the device), directly for the
  // small sections 3-5.
  gb::Mapping file;
  const unsigned char* base = nullptr;
  int fd = -1;
  struct FdGuard {
    int& fd;
    ~FdGuard() {
      if (fd >= 0) ::close(fd);
    }
  } fd_guard{fd};
  uint64_t actual = 0;
  unsigned char hdr[kHeaderBytes];
  if (mmap) {
    file = gb::Mapping(path);
    base = file.data();
    actual = file.size();
  } else {
    fd = ::open(path.c_str(), O_RDONLY);
    if (fd < 0) throw std::runtime_error("cannot open " + path);
    struct stat st {};
    if (::fstat(fd, &st) != 0) throw std::runtime_error("cannot stat " + path);
    actual = static_cast<uint64_t>(st.st_size);
    if (actual < kHeaderBytes) corrupt(path, "file too small for header");
    if (!pread_full(fd, hdr, kHeaderBytes, 0)) corrupt(path, "short read");
  }
  const Fields f = parse_header(mmap ? base : hdr, static_cast<std::size_t>(actual), path);
  auto im = std::make_unique<Impl>(params_of(f));
  im->params.max_elements = f.max_elements;
  const Sizes s = section_bytes(f.count, f.padded_dim, f.M, f.upper_used);
  std::vector<uint8_t> tomb;
  void* dst[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  if (!mmap) {
    if (f.count > 0) im->grow(std::max<std::size_t>(f.count, f.max_elements));
    tomb.resize(f.count);
    im->upper_store.assign(f.upper_used, 0u);
    void* d[6] = {im->vec_store.data(), im->l0_store.data(), im->label_store.data(), im->level_store.data(),
                  tomb.data(), im->upper_store.data()};
    std::copy(d, d + 6, dst);
  }
  hgd_graph_view sizes{};
  sizes.count = f.count;
  sizes.dim = f.dim;
  sizes.padded_dim = f.padded_dim;
  sizes.M = f.M;
  sizes.metric = static_cast<int32_t>(im->params.metric);
  sizes.max_level = f.max_level;
  sizes.entry_point = f.entry;
  constexpr uint64_t kChunk = 32ull << 20;
  hgd_stream* stream = nullptr;
  if (hgd_stream_begin(&sizes, device, im->device_order(), kChunk, &stream) != HGD_OK)
    throw std::runtime_error(std::string("load_to_device: ") + hgd_last_error());
  struct StreamGuard {
    hgd_stream*& s;
    ~StreamGuard() { hgd_stream_abort(s); }
  } stream_guard{stream};
  SectionHash hash;
  uint64_t pos = kHeaderBytes;
  for (int i = 0; i < 6; ++i) {
    unsigned char pad[kSectionAlign];
    const uint64_t gap = f.off[i] - pos;
    if (gap > sizeof pad) corrupt(path, "short read");
    if (mmap) {
      std::memcpy(pad, base + pos, gap);
    } else if (gap && !pread_full(fd, pad, gap, pos)) {
      corrupt(path, "short read");
    }
    for (uint64_t p = 0; p < gap; ++p)
      if (pad[p] != 0) corrupt(path, "non-zero padding");
    for (uint64_t o = 0; o < s.bytes[i]; o += kChunk) {
      const uint64_t len = std::min<uint64_t>(kChunk, s.bytes[i] - o);
      const uint64_t at = f.off[i] + o;
      if (i <= 2) {
        void* buf = nullptr;
        uint64_t cap = 0;
        if (hgd_stream_buffer(stream, &buf, &cap) != HGD_OK)
          throw std::runtime_error(std::string("load_to_device: ") + hgd_last_error());
        if (mmap) std::memcpy(buf, base + at, len);
        else if (!pread_full(fd, buf, len, at)) corrupt(path, "short read");
        hash.feed_part(buf, len, o + len == s.bytes[i], s.bytes[i]);
        if (!mmap) std::memcpy(static_cast<unsigned char*>(dst[i]) + o, buf, len);
        if (hgd_stream_submit(stream, i, o, len) != HGD_OK)
          throw std::runtime_error(std::string("load_to_device: ") + hgd_last_error());
      } else if (mmap) {
        hash.feed_part(base + at, len, o + len == s.bytes[i], s.bytes[i]);
      } else {
        unsigned char* d = static_cast<unsigned char*>(dst[i]) + o;
        if (!pread_full(fd, d, len, at)) corrupt(path, "short read");
        hash.feed_part(d, len, o + len == s.bytes[i], s.bytes[i]);
      }
    }
    if (s.bytes[i] == 0) hash.feed(nullptr, 0);  // an empty section still closes
    pos = f.off[i] + s.bytes[i];
  }
  if (hash.value() != f.payload) corrupt(path, "payload checksum mismatch");
  if (mmap) {
    bind_mapped(*im, f, base);
    check_graph(*im, f, base + f.off[4], path);
    im->mapping = std::move(file);
    im->read_only = true;
  } else {
    im->bind_pointers();
    im->count = f.count;
    im->ef_search = f.ef_search;
    im->upper_used = f.upper_used;
    im->entry_point = f.entry;
    im->max_level = f.max_level;
    im->rng_state = f.rng;
    check_graph(*im, f, tomb.data(), path);
    im->deleted.resize(im->capacity, 0);
  }
  const hgd_graph_view v = im->device_view();
  hgd_graph* g = nullptr;
  hgd_stream* st = stream;
  stream = nullptr;  // finish consumes it, also on failure
  if (hgd_stream_finish(st, &v, &g) != HGD_OK)
    throw std::runtime_error(std::string("load_to_device: ") + hgd_last_error());
  im->device = device;
  hgd_graph_set_launch_mode(g, im->launch_mode);
  im->dev = g;
  im->dev_stale = false;
  return Index(std::move(im));
}

}  // namespace hnsw
