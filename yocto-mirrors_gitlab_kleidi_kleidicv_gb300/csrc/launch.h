// Host-side launch interface of the device kernels.
#pragma once

#include <cuda_runtime.h>

#include "kcv_job.h"

namespace kcv {

// A batched launch of one (mode, size, channels) instantiation: `ntiles`
// tiles of the device job table `jobs`, claimed through *next_tile (0 at
// launch), `grid` CTAs of 128 threads with `smem` bytes of shared memory.
struct BatchLaunch {
  const FilterJob *jobs;
  const BatchTile *tiles;
  int ntiles;
  int *next_tile;
  size_t smem;
  int grid;
};

// Dynamic shared memory the fused kernel needs for `job`'s tiling.
size_t fused_smem_bytes(const FilterJob &job);

// Launches the fused stencil for job.mode / job.ksize / job.channels on
// grid (job.strips, job.row_tiles).  Returns cudaErrorInvalidValue when no
// instantiation exists for the combination.
cudaError_t launch_fused(const FilterJob &job, int *err_flag, cudaStream_t stream);

// Resident CTAs per SM of the fused kernel for `job`'s block size and shared
// memory (0 if no instantiation exists).
int fused_blocks_per_sm(const FilterJob &job);

// Per-family dispatchers (one translation unit each); return false if the
// (mode, ksize, channels) combination is not theirs.  With blocks_per_sm set
// they only report the occupancy instead of launching.
bool launch_fused_binom(const FilterJob &, int *, cudaStream_t, cudaError_t *, int *blocks_per_sm,
                        const BatchLaunch *);
bool launch_fused_sigma_small(const FilterJob &, int *, cudaStream_t, cudaError_t *, int *blocks_per_sm,
                        const BatchLaunch *);
bool launch_fused_sigma_9(const FilterJob &, int *, cudaStream_t, cudaError_t *, int *blocks_per_sm,
                        const BatchLaunch *);
bool launch_fused_sigma_15(const FilterJob &, int *, cudaStream_t, cudaError_t *, int *blocks_per_sm,
                        const BatchLaunch *);
bool launch_fused_sigma_21(const FilterJob &, int *, cudaStream_t, cudaError_t *, int *blocks_per_sm,
                        const BatchLaunch *);
bool launch_fused_sep(const FilterJob &, int *, cudaStream_t, cudaError_t *, int *blocks_per_sm,
                        const BatchLaunch *);
bool launch_fused_blurdown(const FilterJob &, int *, cudaStream_t, cudaError_t *, int *blocks_per_sm,
                        const BatchLaunch *);
bool launch_fused_sobel(const FilterJob &, int *, cudaStream_t, cudaError_t *, int *blocks_per_sm,
                        const BatchLaunch *);

// `rep` is any job of the instantiation (host copy): it selects the kernel.
cudaError_t launch_fused_batch(const FilterJob &rep, const BatchLaunch &b, int *err_flag,
                               cudaStream_t stream);
int fused_batch_blocks_per_sm(const FilterJob &rep, const BatchLaunch &b);

// separable_filter_2d u16 / s16 with 5x5 kernels on one channel
// (csrc/sep16.cu).  sep16_eligible: the job is of that kind, its source rows
// are 16-byte aligned, its destination allows 16-bit stores, and (s16) the
// taps keep every sum exact in fp32.
bool sep16_eligible(const FilterJob &job);
cudaError_t launch_sep16(const FilterJob &job, int sm_count, cudaStream_t stream);

// gaussian_blur_u8 on four channels with generated 3x3 / 5x5 / 7x7 kernels
// summing to 256 (csrc/gauss8.cu).  gauss8_eligible: the job is of that kind
// and its source rows are 4-byte aligned (whole pixels).
bool gauss8_eligible(const FilterJob &job);
// Batch plans (gauss8.cu): the job's Gauss8Job; the resident warps of the
// batched kernel for `ksize`; bands sized for `warps` warps; one launch over
// a device table of n jobs of the same ksize holding `items` warp items.
void gauss8_job(const FilterJob &f, Gauss8Job &j);
int gauss8_batch_warps(int ksize, int sm_count);
void gauss8_size_for_share(Gauss8Job &j, int warps);
cudaError_t launch_gauss8_batch(int ksize, const Gauss8Job *table, int n, long items, int sm_count,
                                cudaStream_t stream);
cudaError_t launch_gauss8(const FilterJob &job, int sm_count, cudaStream_t stream);

// blur_and_downsample_u8 levels (csrc/pyramid.cu): L.phases phases of
// entries, one launch (cooperative when there is more than one phase; the
// barrier counter is cleared on the stream first).
cudaError_t launch_pyramid(const PyrLaunch &L, int sm_count, cudaStream_t stream);
// Fills one level's entry: src (w x h x channels) -> dst ((w+1)/2 x (h+1)/2)
// and its warp items (item_end = the entry's own count), its bands sized for
// `warps` resident warps (pyramid_warps).
void pyr_entry(PyrEntry &e, const uint8_t *src, int64_t src_stride, uint8_t *dst, int64_t dst_stride, int w,
               int h, int channels, int border, int border_value, int warps);
// Resident warps of the pyramid kernel for `channels` on `sm_count` SMs (0 on
// a CUDA failure).
int pyramid_warps(int channels, int sm_count);

// Copies `height` rows of `row_bytes` bytes (any source alignment) into
// `dst`, whose base and stride are multiples of 16 (realign.cu).
cudaError_t launch_realign(const uint8_t *src, int64_t src_stride, uint8_t *dst, int64_t dst_stride,
                           long row_bytes, int height, int sm_count, cudaStream_t stream);

// Generic per-element two-pass Gaussian (arbitrary sizes 11..255, and any
// generated kernel whose weights do not sum to 256).  `scratch` holds the
// u8 intermediate image: width*channels bytes per row, `scratch_stride`
// bytes apart, `height` rows.
cudaError_t launch_generic_gaussian(const GenericJob &job, uint8_t *scratch,
                                    size_t scratch_stride, cudaStream_t stream);

// Loads the two generic kernels on the current device (cudaFuncGetAttributes),
// so that later launches do not trigger CUDA's lazy module loading.
cudaError_t preload_generic_gaussian();

// Median blur: K in {3, 5, 7} for every element type (selection per
// element), K in 9..255 odd for u8 (sliding histograms).
cudaError_t launch_median(const MedianJob &job, cudaStream_t stream);

}  // namespace kcv
