// Host-side internals shared by the C-ABI, batch and serving layers.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <atomic>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <utility>
#include <vector>

#include "../../include/kleidicv_gpu.h"
#include "kcv_job.h"
#include "launch.h"

struct kleidicv_gpu_async;

struct kleidicv_gpu_context {
  int device = 0;
  cudaStream_t stream = nullptr;
  size_t pool_limit = 0;
  std::atomic<size_t> pool_used{0};
  std::atomic<int> fail_allocs{0};
  std::atomic<uint64_t> launches{0};
  int *d_err = nullptr;  // device flag kernels set on a bounded-wait timeout
  int sm_count = 0;
  cudaError_t last_cuda_error = cudaSuccess;
  // Streams and events the batch plans of this context fork onto (created on
  // first use, shared by all plans: every launch orders them through events
  // recorded on `stream`).
  // Tile shape forced on every fused call of the context (the autotuner's
  // knob; threads == 0: the autotune table or the heuristic decide).
  int tune_threads = 0, tune_tile_rows = 0, tune_stage_rows = 0, tune_stages = 0;
  std::mutex branch_mutex;
  std::vector<cudaStream_t> branches;
  std::vector<cudaEvent_t> branch_events;
  cudaEvent_t fork_event = nullptr;
  // Pinned host staging of the scheduler-driven (threaded-API) entries:
  // grow-only, freed with the context.
  void *pinned = nullptr;
  size_t pinned_bytes = 0;
  // Asynchronous threaded-API calls (kleidicv_gpu_thread_*_async): pinned
  // staging buffers kept for reuse, and the completion worker that finishes
  // queued calls in submission order (started on first use, joined by
  // kleidicv_gpu_context_destroy).
  std::mutex pinned_pool_mutex;
  std::vector<std::pair<void *, size_t>> pinned_pool;
  std::mutex async_mutex;
  std::condition_variable async_cv;
  std::deque<kleidicv_gpu_async *> async_queue;
  std::thread async_worker;
  bool async_stop = false;
  // Host-to-device uploads of small tables (batch plans, pyramid entries):
  // a ring of grow-only pinned buffers, each reused once the event recorded
  // after its copy has completed, so no upload waits for the stream to drain.
  struct UploadSlot {
    void *host = nullptr;
    size_t bytes = 0;
    cudaEvent_t done = nullptr;
  };
  static constexpr int kUploadSlots = 8;
  std::mutex upload_mutex;
  UploadSlot upload[kUploadSlots];
  int upload_next = 0;
};

namespace kcv {

bool gaussian_half_kernel(size_t ksize, float sigma, uint8_t *half);

// Tile shape of the fused kernel for one (mode, size, channels, image size).
struct TileShape {
  int threads, tile_rows, stage_rows, stages;
};

// A validated request, ready to be enqueued.
struct Prepared {
  enum Kind { NOTHING, COPY, FUSED, GENERIC } kind = NOTHING;
  FilterJob fused;
  GenericJob generic;
  // COPY (all weight in the centre tap: gaussian_blur_fixed_neon.cpp:565-573)
  const void *src = nullptr;
  size_t src_stride = 0;
  void *dst = nullptr;
  size_t dst_stride = 0;
  size_t row_bytes = 0, rows = 0;
};

kleidicv_error_t prepare_gaussian(const uint8_t *src, size_t src_stride, uint8_t *dst,
                                  size_t dst_stride, size_t width, size_t height,
                                  size_t channels, size_t kernel_width, size_t kernel_height,
                                  float sigma_x, float sigma_y, int border, bool ext,
                                  int border_value, Prepared *out);

// elem: 1 (u8), 2 (u16), 3 (s16).
kleidicv_error_t prepare_separable(int elem, const void *src, size_t src_stride, void *dst,
                                   size_t dst_stride, size_t width, size_t height,
                                   size_t channels, const void *kernel_x, size_t kernel_width,
                                   const void *kernel_y, size_t kernel_height, int border,
                                   bool ext, int border_value, Prepared *out);

kleidicv_error_t prepare_blurdown(const uint8_t *src, size_t src_stride, size_t src_width,
                                  size_t src_height, uint8_t *dst, size_t dst_stride,
                                  size_t channels, int border, bool ext, int border_value,
                                  Prepared *out);

// Median blur checks in the reference's order (median_blur.h:148-193); *work is
// false when a valid call has nothing to compute.  elem: a MedianElem.
kleidicv_error_t validate_median(int elem, size_t es, const void *src, size_t src_stride,
                                 const void *dst, size_t dst_stride, size_t width, size_t height,
                                 size_t channels, size_t kernel_width, size_t kernel_height,
                                 int border, bool *work);

// horizontal: the x derivative (sobel_3x3_horizontal), else the y derivative.
kleidicv_error_t prepare_sobel(bool horizontal, const uint8_t *src, size_t src_stride,
                               int16_t *dst, size_t dst_stride, size_t width, size_t height,
                               size_t channels, Prepared *out);

// Chooses the tile shape (autotune table, else heuristic) and fills the
// derived tiling fields of a FUSED job.  sm_count sizes the grid.
void plan_fused(FilterJob &j, int sm_count);
// Picks tile rows from the kernel's occupancy (after encode_tma).
void finish_plan(FilterJob &j, int sm_count);
TileShape tile_shape_for(const FilterJob &j, int sm_count);
void apply_tile_shape(FilterJob &j, const TileShape &t);
// Builds the TMA descriptor when the source allows it; sets j.use_tma.
void encode_tma(FilterJob &j);

// Enqueues a prepared request on ctx's stream.
kleidicv_error_t execute(kleidicv_gpu_context *ctx, Prepared &p);

// Finishes the context's asynchronous threaded calls and stops its
// completion worker (context destruction).
void shutdown_async(kleidicv_gpu_context *ctx);

// Context helpers.
kleidicv_error_t resolve_context(kleidicv_gpu_context *&ctx);
void *ctx_alloc(kleidicv_gpu_context *ctx, size_t bytes);
void ctx_free(kleidicv_gpu_context *ctx, void *p, size_t bytes);
// Copies `bytes` from host memory `src` to device memory `dst` on the
// context's stream through the pinned upload ring: `src` may be reused as
// soon as the call returns, and the call does not wait for earlier work.
cudaError_t upload_async(kleidicv_gpu_context *ctx, void *dst, const void *src, size_t bytes);
kleidicv_error_t cuda_status(kleidicv_gpu_context *ctx, cudaError_t e);

// Device guard: makes ctx->device current for the calling thread.
struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    if (cudaGetDevice(&prev) == cudaSuccess && prev != dev) cudaSetDevice(dev);
    else prev = -1;
  }
  ~DeviceGuard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
};

}  // namespace kcv
