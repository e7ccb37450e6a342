// Resident CTAs per SM of a kernel, computed once per device.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <mutex>

namespace kcv {

// Raises kernel Kern's dynamic shared-memory limit to `smem` and returns in
// *per_sm how many of its CTAs (`threads` threads, `smem` dynamic bytes) fit
// on one SM (at least 1).  Both are properties of the kernel and the device,
// so the first call on a device asks the runtime and later calls read the
// cached count: a launch makes no attribute or occupancy calls.  Every caller
// of one Kern passes the same threads and smem.  A failure is returned and not
// cached.
template <auto Kern>
cudaError_t resident_ctas_per_sm(int threads, int smem, int *per_sm) {
  constexpr int kDevices = 64;
  static std::atomic<int> cached[kDevices];  // zero-initialised: not yet known
  static std::mutex m;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kDevices) return cudaErrorInvalidDevice;
  int v = cached[dev].load(std::memory_order_acquire);
  if (v == 0) {
    std::lock_guard<std::mutex> lock(m);
    v = cached[dev].load(std::memory_order_relaxed);
    if (v == 0) {
      e = cudaFuncSetAttribute(Kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
      if (e != cudaSuccess) return e;
      int occ = 0;
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, Kern, threads, smem);
      if (e != cudaSuccess) return e;
      v = occ > 1 ? occ : 1;
      cached[dev].store(v, std::memory_order_release);
    }
  }
  *per_sm = v;
  return cudaSuccess;
}

}  // namespace kcv
