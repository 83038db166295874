// smem_limit.cuh -- dynamic shared-memory limits of the kernels (host only).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <unordered_map>

namespace hg {

// Raise a kernel's dynamic shared-memory limit to the device's opt-in
// maximum, once per kernel and device.  The limit is a per-function attribute
// shared by every host thread, so a launcher that set it to its own size could
// lower it under another thread's launch of a larger size; opening it once,
// to the maximum, leaves nothing to race on.  Launches and occupancy queries
// still pass their own size.
inline cudaError_t open_smem_limit(const void* fn) {
  static std::mutex mu;
  static std::unordered_map<const void*, uint64_t> opened;  // kernel -> device bits
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const uint64_t bit = dev < 64 ? (1ull << dev) : 0ull;
  std::lock_guard<std::mutex> lk(mu);
  auto it = opened.find(fn);
  if (bit && it != opened.end() && (it->second & bit)) return cudaSuccess;
  int optin = 0;
  if ((e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev)) != cudaSuccess) return e;
  cudaFuncAttributes fa{};
  if ((e = cudaFuncGetAttributes(&fa, fn)) != cudaSuccess) return e;
  const int dyn = optin - static_cast<int>(fa.sharedSizeBytes);
  if ((e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn)) != cudaSuccess) return e;
  if (bit) opened[fn] |= bit;
  return cudaSuccess;
}

}  // namespace hg
