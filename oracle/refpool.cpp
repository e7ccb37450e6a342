// TEST INFRASTRUCTURE ONLY: linked into oracle/_ref/libkleidicv_ref.so together
// with the reference's own sources, never into the product library.
//
// Two things of ours sit here beside the reference build:
//  * C wrappers (ref_*) over the reference's public entry points of this path,
//    so that Python (ctypes) calls them through plain function symbols whatever
//    form the reference header gives the entry point;
//  * a persistent std::thread pool that implements the reference threaded API's
//    scheduler contract (kleidicv_thread/include/kleidicv_thread/kleidicv_thread.h:42-97):
//    every task index in [0, task_count) runs exactly once, the call returns only
//    after all of them finished, and any failing task makes the call fail.  Unlike
//    the reference's example scheduler (examples/threading/main.cpp:52-86) the
//    threads are created once, so a timed call does not pay thread creation.
#include <sys/prctl.h>

#include <atomic>
#include <condition_variable>
#include <cstddef>
#include <cstdint>
#include <mutex>
#include <thread>
#include <vector>

#include "kleidicv/kleidicv.h"
#include "kleidicv_thread/kleidicv_thread.h"

namespace {

struct Pool {
  std::vector<std::thread> threads;
  std::mutex m;
  std::condition_variable wake, done;
  uint64_t generation = 0;
  unsigned pending = 0;  // workers that have not yet finished the current job
  bool stop = false;
  std::mutex call;  // one job at a time
  kleidicv_thread_callback cb = nullptr;
  void *cb_data = nullptr;
  unsigned count = 0;
  std::atomic<unsigned> next{0};
  std::atomic<int> error{KLEIDICV_OK};
};

void run_tasks(Pool *p) {
  for (;;) {
    unsigned i = p->next.fetch_add(1, std::memory_order_relaxed);
    if (i >= p->count) return;
    kleidicv_error_t e = p->cb(i, i + 1, p->cb_data);
    if (e != KLEIDICV_OK) {
      int ok = KLEIDICV_OK;
      p->error.compare_exchange_strong(ok, static_cast<int>(e));
    }
  }
}

void worker(Pool *p) {
  uint64_t seen = 0;
  std::unique_lock<std::mutex> lk(p->m);
  for (;;) {
    p->wake.wait(lk, [&] { return p->stop || p->generation != seen; });
    if (p->stop) return;
    seen = p->generation;
    lk.unlock();
    run_tasks(p);
    lk.lock();
    if (--p->pending == 0) p->done.notify_all();
  }
}

kleidicv_error_t pool_parallel(kleidicv_thread_callback callback, void *callback_data, void *parallel_data,
                               unsigned task_count) {
  Pool *p = static_cast<Pool *>(parallel_data);
  if (callback == nullptr || p == nullptr) return KLEIDICV_ERROR_NULL_POINTER;
  std::lock_guard<std::mutex> one(p->call);
  {
    std::lock_guard<std::mutex> lk(p->m);
    p->cb = callback;
    p->cb_data = callback_data;
    p->count = task_count;
    p->next.store(0);
    p->error.store(KLEIDICV_OK);
    p->pending = static_cast<unsigned>(p->threads.size());
    ++p->generation;
  }
  p->wake.notify_all();
  run_tasks(p);  // the calling thread works too
  std::unique_lock<std::mutex> lk(p->m);
  p->done.wait(lk, [&] { return p->pending == 0; });
  return static_cast<kleidicv_error_t>(p->error.load());
}

kleidicv_thread_multithreading mt_of(void *pool) { return kleidicv_thread_multithreading{pool_parallel, pool}; }

}  // namespace

extern "C" {

// A pool of `threads` workers in all: threads-1 pool threads plus the caller.
void *ref_pool_create(unsigned threads) {
  Pool *p = new Pool;
  for (unsigned i = 1; i < threads; ++i) p->threads.emplace_back(worker, p);
  return p;
}

void ref_pool_destroy(void *pool) {
  Pool *p = static_cast<Pool *>(pool);
  {
    std::lock_guard<std::mutex> lk(p->m);
    p->stop = true;
  }
  p->wake.notify_all();
  for (auto &t : p->threads) t.join();
  delete p;
}

// SVE vector length of the calling thread in bytes (0 when SVE is absent).
int ref_sve_vector_bytes(void) {
  int r = prctl(51 /* PR_SVE_GET_VL */);
  return r < 0 ? 0 : (r & 0xffff);
}

int ref_gaussian_blur_u8(const uint8_t *src, size_t src_stride, uint8_t *dst, size_t dst_stride, size_t width,
                         size_t height, size_t channels, size_t kw, size_t kh, float sx, float sy, int border) {
  return kleidicv_gaussian_blur_u8(src, src_stride, dst, dst_stride, width, height, channels, kw, kh, sx, sy,
                                   static_cast<kleidicv_border_type_t>(border));
}

int ref_separable_filter_2d_u8(const uint8_t *src, size_t src_stride, uint8_t *dst, size_t dst_stride,
                               size_t width, size_t height, size_t channels, const uint8_t *kx, size_t kw,
                               const uint8_t *ky, size_t kh, int border) {
  return kleidicv_separable_filter_2d_u8(src, src_stride, dst, dst_stride, width, height, channels, kx, kw, ky, kh,
                                         static_cast<kleidicv_border_type_t>(border));
}

int ref_separable_filter_2d_u16(const uint16_t *src, size_t src_stride, uint16_t *dst, size_t dst_stride,
                                size_t width, size_t height, size_t channels, const uint16_t *kx, size_t kw,
                                const uint16_t *ky, size_t kh, int border) {
  return kleidicv_separable_filter_2d_u16(src, src_stride, dst, dst_stride, width, height, channels, kx, kw, ky,
                                          kh, static_cast<kleidicv_border_type_t>(border));
}

int ref_blur_and_downsample_u8(const uint8_t *src, size_t src_stride, size_t width, size_t height, uint8_t *dst,
                               size_t dst_stride, size_t channels, int border) {
  return kleidicv_blur_and_downsample_u8(src, src_stride, width, height, dst, dst_stride, channels,
                                         static_cast<kleidicv_border_type_t>(border));
}

int ref_sobel_3x3_horizontal_s16_u8(const uint8_t *src, size_t src_stride, int16_t *dst, size_t dst_stride,
                                    size_t width, size_t height, size_t channels) {
  return kleidicv_sobel_3x3_horizontal_s16_u8(src, src_stride, dst, dst_stride, width, height, channels);
}

int ref_sobel_3x3_vertical_s16_u8(const uint8_t *src, size_t src_stride, int16_t *dst, size_t dst_stride,
                                  size_t width, size_t height, size_t channels) {
  return kleidicv_sobel_3x3_vertical_s16_u8(src, src_stride, dst, dst_stride, width, height, channels);
}

#define REF_MEDIAN(suffix, T)                                                                                  \
  int ref_median_blur_##suffix(const T *src, size_t src_stride, T *dst, size_t dst_stride, size_t width,      \
                               size_t height, size_t channels, size_t kw, size_t kh, int border) {           \
    return kleidicv_median_blur_##suffix(src, src_stride, dst, dst_stride, width, height, channels, kw, kh,    \
                                         static_cast<kleidicv_border_type_t>(border));                        \
  }
REF_MEDIAN(s8, int8_t)
REF_MEDIAN(u8, uint8_t)
REF_MEDIAN(u16, uint16_t)
REF_MEDIAN(s16, int16_t)
REF_MEDIAN(u32, uint32_t)
REF_MEDIAN(s32, int32_t)
REF_MEDIAN(f32, float)
#undef REF_MEDIAN

// LK pyramid: build, read one level (image or Scharr pairs) and release.
int ref_lk_pyramid_build(void **out, const uint8_t *src, size_t src_stride, size_t width, size_t height,
                         size_t channels, size_t levels, size_t window_w, size_t window_h) {
  kleidicv_optical_flow_pyr_lk_pyramid_t *p = nullptr;
  kleidicv_error_t e = kleidicv_build_optical_flow_pyr_lk_pyramid(&p, src, src_stride, width, height, channels,
                                                                  levels, window_w, window_h);
  *out = p;
  return e;
}

int ref_lk_pyramid_level_count(const void *pyr, size_t *count) {
  return kleidicv_optical_flow_pyr_lk_pyramid_get_level_count(
      static_cast<const kleidicv_optical_flow_pyr_lk_pyramid_t *>(pyr), count);
}

int ref_lk_pyramid_image_level(const void *pyr, size_t level, const uint8_t **data, size_t *stride, size_t *w,
                               size_t *h) {
  return kleidicv_optical_flow_pyr_lk_pyramid_get_image_level(
      static_cast<const kleidicv_optical_flow_pyr_lk_pyramid_t *>(pyr), level, data, stride, w, h);
}

int ref_lk_pyramid_scharr_level(const void *pyr, size_t level, const int16_t **data, size_t *stride, size_t *w,
                                size_t *h) {
  return kleidicv_optical_flow_pyr_lk_pyramid_get_scharr_level(
      static_cast<const kleidicv_optical_flow_pyr_lk_pyramid_t *>(pyr), level, data, stride, w, h);
}

int ref_lk_pyramid_release(void *pyr) {
  return kleidicv_optical_flow_pyr_lk_pyramid_release(static_cast<kleidicv_optical_flow_pyr_lk_pyramid_t *>(pyr));
}

// Threaded twins, scheduled on a pool from ref_pool_create.
int ref_thread_gaussian_blur_u8(void *pool, const uint8_t *src, size_t src_stride, uint8_t *dst, size_t dst_stride,
                                size_t width, size_t height, size_t channels, size_t kw, size_t kh, float sx,
                                float sy, int border) {
  return kleidicv_thread_gaussian_blur_u8(src, src_stride, dst, dst_stride, width, height, channels, kw, kh, sx, sy,
                                          static_cast<kleidicv_border_type_t>(border), mt_of(pool));
}

int ref_thread_separable_filter_2d_u8(void *pool, const uint8_t *src, size_t src_stride, uint8_t *dst,
                                      size_t dst_stride, size_t width, size_t height, size_t channels,
                                      const uint8_t *kx, size_t kw, const uint8_t *ky, size_t kh, int border) {
  return kleidicv_thread_separable_filter_2d_u8(src, src_stride, dst, dst_stride, width, height, channels, kx, kw,
                                                ky, kh, static_cast<kleidicv_border_type_t>(border), mt_of(pool));
}

int ref_thread_separable_filter_2d_u16(void *pool, const uint16_t *src, size_t src_stride, uint16_t *dst,
                                       size_t dst_stride, size_t width, size_t height, size_t channels,
                                       const uint16_t *kx, size_t kw, const uint16_t *ky, size_t kh, int border) {
  return kleidicv_thread_separable_filter_2d_u16(src, src_stride, dst, dst_stride, width, height, channels, kx, kw,
                                                 ky, kh, static_cast<kleidicv_border_type_t>(border), mt_of(pool));
}

int ref_thread_blur_and_downsample_u8(void *pool, const uint8_t *src, size_t src_stride, size_t width,
                                      size_t height, uint8_t *dst, size_t dst_stride, size_t channels, int border) {
  return kleidicv_thread_blur_and_downsample_u8(src, src_stride, width, height, dst, dst_stride, channels,
                                                static_cast<kleidicv_border_type_t>(border), mt_of(pool));
}

int ref_thread_sobel_3x3_horizontal_s16_u8(void *pool, const uint8_t *src, size_t src_stride, int16_t *dst,
                                           size_t dst_stride, size_t width, size_t height, size_t channels) {
  return kleidicv_thread_sobel_3x3_horizontal_s16_u8(src, src_stride, dst, dst_stride, width, height, channels,
                                                     mt_of(pool));
}

int ref_thread_median_blur_u8(void *pool, const uint8_t *src, size_t src_stride, uint8_t *dst, size_t dst_stride,
                              size_t width, size_t height, size_t channels, size_t kw, size_t kh, int border) {
  return kleidicv_thread_median_blur_u8(src, src_stride, dst, dst_stride, width, height, channels, kw, kh,
                                        static_cast<kleidicv_border_type_t>(border), mt_of(pool));
}

}  // extern "C"
