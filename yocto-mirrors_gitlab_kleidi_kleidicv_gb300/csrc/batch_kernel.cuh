// Batched persistent kernel: for one (mode, size, channels) instantiation it
// walks a device-side work-list of tiles drawn from many jobs (images of
// uneven sizes).  CTAs claim tiles with an atomic counter, so large and small
// images balance across the GPU; the job table (FilterJob, including its
// tensor maps) lives in global memory.  A batch launches one such kernel per
// instantiation it needs, concurrently.
//
// Every tile may use a different ring shape, so the mbarriers are
// invalidated and re-initialised between tiles, once every warp has finished
// the previous tile (all of its copies have landed and been consumed).
#pragma once

#include "launch.h"
#include "sepfused.cuh"

namespace kcv {

template <int MODE, int K, int C, bool NARROW>
__global__ void __launch_bounds__(128, (K >= 15 ? 2 : 4))
    batch_kernel(const FilterJob *__restrict__ jobs, const BatchTile *__restrict__ tiles,
                 int ntiles, int *next_tile, int *err_flag) {
  extern __shared__ __align__(128) uint8_t smem[];
  __shared__ int s_tile;
  uint64_t *bars = reinterpret_cast<uint64_t *>(smem);
  int live_bars = 0;  // mbarriers currently initialised (thread 0 only)
  bool timed_out = false;
  for (;;) {
    // Every warp has finished the previous tile here: its copies have landed
    // and been consumed, so the barriers may be re-initialised.
    __syncthreads();
    if (threadIdx.x == 0) s_tile = atomicAdd(next_tile, 1);
    __syncthreads();
    const int t = s_tile;
    if (t >= ntiles) break;
    const BatchTile bt = tiles[t];
    const FilterJob &j = jobs[bt.job];
    if (j.use_tma) {
      if (threadIdx.x == 0) {
        for (int b = 0; b < live_bars; ++b) mbar_inval(&bars[b]);
        prefetch_tensormap(&j.tmap);
        prefetch_tensormap(&j.tmap_row);
        const int warps = blockDim.x / 32;
        for (int s = 0; s < j.stages; ++s) {
          mbar_init(&bars[s], 1);
          mbar_init(&bars[j.stages + s], warps);
        }
        live_bars = 2 * j.stages;
        fence_mbar_init();
      }
      __syncthreads();
    }
    uint32_t gstage = 0;
    const TmaMaps maps{&j.tmap, &j.tmap_row, &j.tmap_wrap, &j.tmap_wrap_row};
    // Without the aligned-block stores: the batched kernels measured faster
    // without that code, unaligned destinations included.
    run_tile<MODE, K, C, NARROW, false>(j, maps, bt.strip, bt.band, smem, gstage, err_flag, timed_out);
  }
}

}  // namespace kcv
