// bruteforce.cu -- exact k-NN (BruteForceIndex, reference src/brute_force.cpp:34-69).
//
// Rows are stored sorted by label, so the key (order-preserving distance
// bits << 32 | row) orders exactly like the reference's (distance, label)
// heap.  Distances use the reference kernel's order over `dim` (not the
// padded dimension), the host's as the reference picks it: AVX-512 (64-float
// blocks into acc0..acc3, 16-float blocks into acc0, the masked remainder
// into acc1) or NEON (16-float blocks into four 4-lane accumulators, 4-float
// blocks into acc0, a fused scalar tail); see bf_common.cuh.
//
// One block = 16 warps x QT queries.  Each warp scans an interleaved share
// of the rows with the QT queries held in registers and keeps, per query, a
// sorted top-k list in shared memory; the block then merges its 16 lists per
// query with a bitonic sort and writes the first k.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <numeric>
#include <string>
#include <vector>

#include "bf_common.cuh"
#include "bf_mma.h"
#include "smem_limit.cuh"
#include "hnswgpu_device.h"

namespace hg {
void set_last_error(const std::string& msg);
}

namespace {

constexpr int kWarps = 16;
constexpr uint32_t kMaxK = 256;
using namespace hg::bf;

struct BfParams {
  const float* rows;       // n x dp, sorted by label
  const uint64_t* labels;  // n, sorted
  const uint32_t* allow;   // n bits over sorted rows, or null
  const float* queries;    // nq x dim raw
  const float* inv;        // cosine: per query 1/||q|| or null
  uint32_t n, dim, dp, nq, k;
  int32_t neon;            // distance order: 1 NEON, 0 AVX-512
  void* out;
};

template <int S, int QT, bool L2>
__global__ void __launch_bounds__(kWarps * 32) bf_kernel(BfParams P) {
  extern __shared__ __align__(16) unsigned char smem[];
  uint64_t* lists = reinterpret_cast<uint64_t*>(smem);  // [warp][QT][k]
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const uint32_t q0 = blockIdx.x * QT;
  const BfOrder o = bf_order(P.dim, P.neon != 0);
  const uint32_t k = P.k;
  float qr[QT][S];
#pragma unroll
  for (int t = 0; t < QT; ++t) {
    const uint32_t q = q0 + t < P.nq ? q0 + t : q0;
    const float* raw = P.queries + static_cast<size_t>(q) * P.dim;
    const float inv = P.inv ? P.inv[q] : 1.0f;
#pragma unroll
    for (int i = 0; i < S; ++i) {
      const int e = bslot(o, i, lane);
      const float v = e >= 0 ? raw[e] : 0.0f;
      qr[t][i] = P.inv ? __fmul_rn(v, inv) : v;
    }
  }
  uint64_t* my = lists + static_cast<size_t>(w) * QT * k;
  int cnt[QT];
#pragma unroll
  for (int t = 0; t < QT; ++t) cnt[t] = 0;
  for (uint32_t r = w; r < P.n; r += kWarps) {
    if (P.allow && !((P.allow[r >> 5] >> (r & 31)) & 1u)) continue;
    const float* row = P.rows + static_cast<size_t>(r) * P.dp;
    float x[S];
#pragma unroll
    for (int i = 0; i < S; ++i) {
      const int e = bslot(o, i, lane);
      x[i] = e >= 0 ? __ldg(row + e) : 0.0f;
    }
#pragma unroll
    for (int t = 0; t < QT; ++t) {
      const float d = bdist<S, L2>(x, qr[t], o, lane);
      const uint64_t key = (static_cast<uint64_t>(okey(d)) << 32) | r;
      uint64_t* L = my + static_cast<size_t>(t) * k;
      const int c = cnt[t];
      if (c == static_cast<int>(k) && key >= L[k - 1]) continue;
      // insert: position = number of entries < key
      int pos = 0;
      for (int base = 0; base < c; base += 32) {
        const bool lt = base + lane < c && L[base + lane] < key;
        pos += __popc(__ballot_sync(kFull, lt));
      }
      const int last = c < static_cast<int>(k) ? c : static_cast<int>(k) - 1;
      for (int top = last; top > pos; top -= 32) {
        const int p = top - 1 - lane;  // move p -> p + 1
        uint64_t v = 0;
        const bool mv = p >= pos;
        if (mv) v = L[p];
        __syncwarp();
        if (mv) L[p + 1] = v;
        __syncwarp();
      }
      if (lane == 0) L[pos] = key;
      __syncwarp();
      cnt[t] = c < static_cast<int>(k) ? c + 1 : c;
    }
  }
  // pad short lists, then merge the 16 lists of each query
#pragma unroll
  for (int t = 0; t < QT; ++t)
    for (int i = cnt[t] + lane; i < static_cast<int>(k); i += 32) my[static_cast<size_t>(t) * k + i] = ~0ull;
  __syncthreads();
  uint64_t* tmp = lists + static_cast<size_t>(kWarps) * QT * k;  // kWarps*k rounded to pow2
  int p2 = 1;
  while (p2 < kWarps * static_cast<int>(k)) p2 <<= 1;
  for (int t = 0; t < QT; ++t) {
    const uint32_t q = q0 + t;
    if (q >= P.nq) break;
    for (int i = threadIdx.x; i < p2; i += blockDim.x) {
      const int ww = i / static_cast<int>(k), j = i % static_cast<int>(k);
      tmp[i] = ww < kWarps ? lists[(static_cast<size_t>(ww) * QT + t) * k + j] : ~0ull;
    }
    __syncthreads();
    for (int kk = 2; kk <= p2; kk <<= 1) {
      for (int j = kk >> 1; j > 0; j >>= 1) {
        for (int i = threadIdx.x; i < p2; i += blockDim.x) {
          const int l = i ^ j;
          if (l > i) {
            const uint64_t a = tmp[i], b = tmp[l];
            const bool up = (i & kk) == 0;
            if ((a > b) == up) {
              tmp[i] = b;
              tmp[l] = a;
            }
          }
        }
        __syncthreads();
      }
    }
    Rec* row = static_cast<Rec*>(P.out) + static_cast<size_t>(q) * k;
    for (uint32_t j = threadIdx.x; j < k; j += blockDim.x) {
      const uint64_t key = tmp[j];
      Rec o;
      if (key == ~0ull) {
        o.label = ~0ull;
        o.dist = __int_as_float(0x7f800000);
      } else {
        o.label = P.labels[static_cast<uint32_t>(key)];
        o.dist = key_dist(key);
      }
      o.zero = 0;
      row[j] = o;
    }
    __syncthreads();
  }
}

__global__ void bf_inv_norm(const float* qs, uint32_t nq, uint32_t dim, float* out) {
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq) return;
  double norm = 0.0;
  for (uint32_t i = 0; i < dim; ++i) {
    const double v = static_cast<double>(qs[static_cast<size_t>(q) * dim + i]);
    norm = __dadd_rn(norm, __dmul_rn(v, v));
  }
  out[q] = norm > 0.0 ? __double2float_rn(1.0 / sqrt(norm)) : 1.0f;
}

__global__ void bf_translate(const uint64_t* words, uint64_t num_bits, const uint64_t* labels, uint32_t n,
                             uint32_t* out) {
  const uint32_t wd = blockIdx.x * blockDim.x + threadIdx.x;
  if (wd >= (n + 31) / 32) return;
  uint32_t bits = 0;
  for (uint32_t b = 0; b < 32; ++b) {
    const uint64_t r = static_cast<uint64_t>(wd) * 32 + b;
    if (r >= n) break;
    const uint64_t l = labels[r];
    if (l < num_bits && ((words[l >> 6] >> (l & 63)) & 1ull)) bits |= 1u << b;
  }
  out[wd] = bits;
}

template <int S, int QT, bool L2>
cudaError_t bf_launch(const BfParams& P, cudaStream_t st) {
  int p2 = 1;
  while (p2 < kWarps * static_cast<int>(P.k)) p2 <<= 1;
  const size_t smem = (static_cast<size_t>(kWarps) * QT * P.k + p2) * 8;
  auto* fn = bf_kernel<S, QT, L2>;
  cudaError_t e = hg::open_smem_limit(reinterpret_cast<const void*>(fn));
  if (e != cudaSuccess) return e;
  fn<<<(P.nq + QT - 1) / QT, kWarps * 32, smem, st>>>(P);
  return cudaGetLastError();
}

template <bool L2>
cudaError_t bf_dispatch(const BfParams& P, cudaStream_t st) {
  const int S = bf_slots(P.dim, P.neon != 0);
  const bool big_k = P.k > 64;
  if (S <= 6) return big_k ? bf_launch<6, 1, L2>(P, st) : bf_launch<6, 4, L2>(P, st);
  if (S <= 10) return big_k ? bf_launch<10, 1, L2>(P, st) : bf_launch<10, 2, L2>(P, st);
  if (S <= 18) return bf_launch<18, 1, L2>(P, st);
  if (S <= 34) return bf_launch<34, 1, L2>(P, st);
  if (S <= 70) return bf_launch<70, 1, L2>(P, st);  // the NEON order of rows above 512 elements
  return cudaErrorInvalidValue;
}

}  // namespace

struct hgd_flat {
  int device = 0, metric = 0;
  uint32_t n = 0, dim = 0, dp = 0;
  float* rows = nullptr;
  uint64_t* labels = nullptr;
  std::vector<uint64_t> orig_of_sorted;  // sorted row -> insertion index
  cudaStream_t stream = nullptr;
  hg::bfm::Store* tensor = nullptr;  // FP16 copy for the tensor-core path (built on first use)
  int path = HGD_BF_AUTO;
  int last_path = 0;
  bool neon = false;  // distance order
};

extern "C" {

int hgd_flat_upload(const float* prepared, const uint64_t* labels, uint64_t n, uint64_t dim, int metric, int device,
                    int order, hgd_flat** out) {
  if (!out || (n && (!prepared || !labels))) return (hg::set_last_error("hgd_flat_upload: null argument"), HGD_EINVAL);
  if (order != HGD_ORDER_AVX512 && order != HGD_ORDER_NEON)
    return (hg::set_last_error("brute force: the GPU implements the AVX-512 and NEON orders only"), HGD_EINVAL);
  if (n >= 0xFFFFFFFFull || dim == 0 || dim > 1056)
    return (hg::set_last_error("brute force: unsupported size"), HGD_EINVAL);
  auto* f = new hgd_flat();
  f->device = device;
  f->metric = metric;
  f->n = static_cast<uint32_t>(n);
  f->dim = static_cast<uint32_t>(dim);
  f->dp = (f->dim + 15) / 16 * 16;
  f->neon = order == HGD_ORDER_NEON;
  std::vector<uint64_t> order_idx(n);
  std::iota(order_idx.begin(), order_idx.end(), 0);
  std::stable_sort(order_idx.begin(), order_idx.end(), [&](uint64_t a, uint64_t b) { return labels[a] < labels[b]; });
  std::vector<float> rows(static_cast<size_t>(n) * f->dp, 0.0f);
  std::vector<uint64_t> lab(n);
  for (uint64_t i = 0; i < n; ++i) {
    std::copy(prepared + order_idx[i] * dim, prepared + order_idx[i] * dim + dim, rows.begin() + i * f->dp);
    lab[i] = labels[order_idx[i]];
  }
  f->orig_of_sorted = std::move(order_idx);
  auto bad = [&](cudaError_t e) {
    hg::set_last_error(std::string("hgd_flat_upload: ") + cudaGetErrorString(e));
    hgd_flat_free(f);
    return e == cudaErrorMemoryAllocation ? HGD_ENOMEM : HGD_ECUDA;
  };
  cudaError_t e;
  if ((e = cudaSetDevice(device)) != cudaSuccess) return bad(e);
  if ((e = cudaStreamCreateWithFlags(&f->stream, cudaStreamNonBlocking)) != cudaSuccess) return bad(e);
  if ((e = cudaMalloc(&f->rows, std::max<size_t>(rows.size() * 4, 16))) != cudaSuccess) return bad(e);
  if ((e = cudaMalloc(&f->labels, std::max<size_t>(n * 8, 16))) != cudaSuccess) return bad(e);
  if (n) {
    if ((e = cudaMemcpy(f->rows, rows.data(), rows.size() * 4, cudaMemcpyHostToDevice)) != cudaSuccess) return bad(e);
    if ((e = cudaMemcpy(f->labels, lab.data(), n * 8, cudaMemcpyHostToDevice)) != cudaSuccess) return bad(e);
  }
  *out = f;
  return HGD_OK;
}

void hgd_flat_free(hgd_flat* f) {
  if (!f) return;
  cudaSetDevice(f->device);
  if (f->rows) cudaFree(f->rows);
  if (f->labels) cudaFree(f->labels);
  hg::bfm::store_free(f->tensor);
  if (f->stream) cudaStreamDestroy(f->stream);
  delete f;
}

int hgd_flat_set_path(hgd_flat* f, int path) {
  if (!f || path < HGD_BF_AUTO || path > HGD_BF_TENSOR)
    return (hg::set_last_error("hgd_flat_set_path: bad argument"), HGD_EINVAL);
  f->path = path;
  return HGD_OK;
}

int hgd_flat_last_path(const hgd_flat* f) { return f ? f->last_path : 0; }

int hgd_bruteforce(hgd_flat* f, const float* queries, uint64_t nq, uint32_t k, const hgd_bitset* filter, void* out,
                   void* stream) {
  if (!f || !queries || !out) return (hg::set_last_error("hgd_bruteforce: null argument"), HGD_EINVAL);
  if (k == 0) return (hg::set_last_error("search: k must be > 0"), HGD_EINVAL);
  if (k > kMaxK) return (hg::set_last_error("brute force: k above 256 is not supported"), HGD_EINVAL);
  const bool tensor_ok = hg::bfm::supported(f->dim, k);
  if (f->path == HGD_BF_TENSOR && !tensor_ok)
    return (hg::set_last_error("brute force: the tensor path needs dim <= 1024 and k <= 256"), HGD_EINVAL);
  const bool use_tensor = f->path != HGD_BF_SCAN && tensor_ok;
  if (nq == 0) return HGD_OK;
  cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : f->stream;
  float *dq = nullptr, *dinv = nullptr;
  uint32_t* dallow = nullptr;
  uint64_t* dwords = nullptr;
  void* dout = nullptr;
  int rc = HGD_OK;
  auto check = [&](cudaError_t e) {
    if (e != cudaSuccess && rc == HGD_OK) {
      hg::set_last_error(std::string("hgd_bruteforce: ") + cudaGetErrorString(e));
      rc = e == cudaErrorMemoryAllocation ? HGD_ENOMEM : HGD_ECUDA;
    }
    return e == cudaSuccess;
  };
  do {
    if (!check(cudaSetDevice(f->device))) break;
    if (!check(cudaMalloc(&dq, nq * f->dim * 4))) break;
    if (!check(cudaMalloc(&dout, nq * k * 16))) break;
    if (!check(cudaMemcpyAsync(dq, queries, nq * f->dim * 4, cudaMemcpyHostToDevice, st))) break;
    if (f->metric == HGD_METRIC_COSINE) {
      if (!check(cudaMalloc(&dinv, nq * 4))) break;
      bf_inv_norm<<<static_cast<unsigned>((nq + 127) / 128), 128, 0, st>>>(dq, static_cast<uint32_t>(nq), f->dim,
                                                                           dinv);
      if (!check(cudaGetLastError())) break;
    }
    if (filter) {
      const uint32_t words32 = (f->n + 31) / 32 + 1;
      if (!check(cudaMalloc(&dallow, words32 * 4))) break;
      if (filter->label_space) {
        const uint64_t w64 = (filter->num_bits + 63) / 64;
        if (!check(cudaMalloc(&dwords, std::max<uint64_t>(w64, 1) * 8))) break;
        if (w64 && !check(cudaMemcpyAsync(dwords, filter->words, w64 * 8, cudaMemcpyHostToDevice, st))) break;
        bf_translate<<<(words32 + 255) / 256, 256, 0, st>>>(dwords, filter->num_bits, f->labels, f->n, dallow);
        if (!check(cudaGetLastError())) break;
      } else {
        std::vector<uint32_t> bits(words32, 0);
        for (uint32_t r = 0; r < f->n; ++r) {
          const uint64_t o = f->orig_of_sorted[r];
          if (o < filter->num_bits && ((filter->words[o >> 6] >> (o & 63)) & 1ull)) bits[r >> 5] |= 1u << (r & 31);
        }
        if (!check(cudaMemcpyAsync(dallow, bits.data(), words32 * 4, cudaMemcpyHostToDevice, st))) break;
        if (!check(cudaStreamSynchronize(st))) break;
      }
    }
    if (use_tensor) {
      hg::bfm::Rows R{f->rows, f->labels, f->n, f->dim, f->dp, f->metric, f->neon ? 1 : 0};
      std::string err;
      if (!f->tensor && !check(hg::bfm::store_create(R, st, &f->tensor, &err))) {
        hg::set_last_error(err);
        break;
      }
      bool redo = false;
      const cudaError_t e = hg::bfm::search(f->tensor, R, dq, dinv, static_cast<uint32_t>(nq), k, dallow, dout, st,
                                            &redo, &err);
      if (e != cudaSuccess) {
        check(e);
        hg::set_last_error(err);
        break;
      }
      if (!redo) {
        f->last_path = HGD_BF_TENSOR;
        if (!check(cudaMemcpyAsync(out, dout, nq * k * 16, cudaMemcpyDeviceToHost, st))) break;
        check(cudaStreamSynchronize(st));
        break;
      }
      // some query kept more near-ties than the buffers hold: the scan answers the batch
    }
    f->last_path = HGD_BF_SCAN;
    BfParams P{};
    P.rows = f->rows;
    P.labels = f->labels;
    P.allow = dallow;
    P.queries = dq;
    P.inv = dinv;
    P.n = f->n;
    P.dim = f->dim;
    P.dp = f->dp;
    P.nq = static_cast<uint32_t>(nq);
    P.k = k;
    P.neon = f->neon ? 1 : 0;
    P.out = dout;
    if (!check(f->metric == HGD_METRIC_L2 ? bf_dispatch<true>(P, st) : bf_dispatch<false>(P, st))) break;
    if (!check(cudaMemcpyAsync(out, dout, nq * k * 16, cudaMemcpyDeviceToHost, st))) break;
    check(cudaStreamSynchronize(st));
  } while (false);
  cudaStreamSynchronize(st);
  if (dq) cudaFree(dq);
  if (dinv) cudaFree(dinv);
  if (dallow) cudaFree(dallow);
  if (dwords) cudaFree(dwords);
  if (dout) cudaFree(dout);
  return rc;
}

}  // extern "C"
