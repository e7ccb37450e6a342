// Helpers shared by the fused-kernel instantiation units.
#pragma once

#include <algorithm>
#include <atomic>
#include <mutex>

#include "launch.h"
#include "batch_kernel.cuh"

namespace kcv {

constexpr int kMaxDevices = 64;

// Raises kernel Kern's dynamic shared-memory limit once per device (the
// attribute is per device); safe under concurrent first calls.  A failed
// attempt is not remembered: the next launch on that device tries again.  The
// kernel is a template argument so that every kernel has its own flags.
template <auto Kern>
cudaError_t allow_large_smem() {
  static std::atomic<bool> done[kMaxDevices];  // zero-initialised: false
  static std::mutex m;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  if (done[dev].load(std::memory_order_acquire)) return cudaSuccess;
  std::lock_guard<std::mutex> lock(m);
  if (done[dev].load(std::memory_order_relaxed)) return cudaSuccess;
  e = cudaFuncSetAttribute(Kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
  if (e == cudaSuccess) done[dev].store(true, std::memory_order_release);
  return e;
}

// Plain launch of `job` (batch == nullptr) or of the batched kernel of the
// same instantiation over batch->tiles.  With blocks_per_sm set, only reports
// the occupancy.
template <int MODE, int K, int C, bool NARROW>
cudaError_t launch_one(const FilterJob &job, int *err_flag, cudaStream_t stream,
                       int *blocks_per_sm, const BatchLaunch *batch) {
  if (batch) {
    auto kern = batch_kernel<MODE, K, C, NARROW>;
    if (cudaError_t e = allow_large_smem<batch_kernel<MODE, K, C, NARROW>>(); e != cudaSuccess) return e;
    if (blocks_per_sm) {
      // Cached per instantiation and device for the last shared-memory size asked.
      static size_t cached_smem[kMaxDevices];
      static int cached_occ[kMaxDevices];
      static bool valid[kMaxDevices];
      static std::mutex m;
      int dev = 0;
      if (cudaError_t e = cudaGetDevice(&dev); e != cudaSuccess) return e;
      if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
      std::lock_guard<std::mutex> lock(m);
      if (!valid[dev] || cached_smem[dev] != batch->smem) {
        cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&cached_occ[dev], kern, 128, batch->smem);
        if (e != cudaSuccess) return e;
        cached_smem[dev] = batch->smem;
        valid[dev] = true;
      }
      *blocks_per_sm = cached_occ[dev];
      return cudaSuccess;
    }
    kern<<<static_cast<unsigned>(batch->grid), 128, batch->smem, stream>>>(
        batch->jobs, batch->tiles, batch->ntiles, batch->next_tile, err_flag);
    return cudaGetLastError();
  }
  const SmemLayout L = smem_layout(MODE, K, C, job.threads, job.halo_chunks, job.box_lbw,
                                   job.stage_rows, job.stages, job.use_tma != 0,
                                   job.border == BORDER_WRAP);
  auto kern = sepfused_kernel<MODE, K, C, NARROW>;
  if (cudaError_t e = allow_large_smem<sepfused_kernel<MODE, K, C, NARROW>>(); e != cudaSuccess)
    return e;
  // One wave of persistent CTAs: as many as fit on the device at once.
  int per_sm = 0, dev = 0, sms = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, job.threads, L.total);
  if (e != cudaSuccess) return e;
  if (blocks_per_sm) {
    *blocks_per_sm = per_sm;
    return cudaSuccess;
  }
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long tiles = static_cast<long>(job.strips) * job.row_tiles;
  const long grid = std::max(1L, std::min(tiles, static_cast<long>(std::max(per_sm, 1)) * sms));
  // Programmatic stream serialization: this launch may begin while the
  // previous kernel on the stream drains (the kernel waits for it before
  // touching memory).
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(static_cast<unsigned>(grid));
  cfg.blockDim = dim3(static_cast<unsigned>(job.threads));
  cfg.dynamicSmemBytes = L.total;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, job, err_flag);
}

template <int MODE, int K, bool NARROW>
bool dispatch_channels_n(const FilterJob &job, int *err, cudaStream_t s, cudaError_t *out,
                         int *blocks_per_sm, const BatchLaunch *b) {
  switch (job.channels) {
    case 1: *out = launch_one<MODE, K, 1, NARROW>(job, err, s, blocks_per_sm, b); return true;
    case 2: *out = launch_one<MODE, K, 2, NARROW>(job, err, s, blocks_per_sm, b); return true;
    case 3: *out = launch_one<MODE, K, 3, NARROW>(job, err, s, blocks_per_sm, b); return true;
    case 4: *out = launch_one<MODE, K, 4, NARROW>(job, err, s, blocks_per_sm, b); return true;
  }
  return false;
}

// Separable modes have a narrow-tap instantiation (job.narrow); the Gaussian
// and blur-and-downsample arithmetic is narrow by construction.
template <int MODE, int K>
bool dispatch_channels(const FilterJob &job, int *err, cudaStream_t s, cudaError_t *out,
                       int *blocks_per_sm, const BatchLaunch *b) {
  if constexpr (MODE == MODE_SEP_U8 || MODE == MODE_SEP_U16 || MODE == MODE_SEP_S16) {
    if (job.narrow) return dispatch_channels_n<MODE, K, true>(job, err, s, out, blocks_per_sm, b);
  }
  return dispatch_channels_n<MODE, K, false>(job, err, s, out, blocks_per_sm, b);
}

}  // namespace kcv
