/*
 * kleidicv_gpu_thread.h -- the threaded API of KleidiCV's separable-filter
 * path over the GPU, driven by the caller's scheduler.
 *
 * KleidiCV's threaded API (kleidicv_thread/include/kleidicv_thread/
 * kleidicv_thread.h:42-97, 457-531) takes HOST images and a caller-provided
 * scheduler (`kleidicv_thread_multithreading mt`): the library cuts the work
 * into task ranges and asks the scheduler to run them, then returns when the
 * result is in `dst`.  The functions below have exactly those parameter
 * lists and that contract, with the filtering done on the GPU:
 *
 *   kleidicv_gpu_thread_gaussian_blur_u8          kleidicv_thread.h:459-463
 *   kleidicv_gpu_thread_separable_filter_2d_u8    kleidicv_thread.h:467-471
 *   kleidicv_gpu_thread_separable_filter_2d_u16   kleidicv_thread.h:475-479
 *   kleidicv_gpu_thread_blur_and_downsample_u8    kleidicv_thread.h:482-485
 *   kleidicv_gpu_thread_sobel_3x3_{horizontal,vertical}_s16_u8
 *                                                 kleidicv_thread.h:489-492, 528-531
 *   kleidicv_gpu_thread_median_blur_{s8,u8,u16,s16,u32,s32,f32}
 *                                                 kleidicv_thread.h:496-524
 *
 * The scheduler's tasks are row stripes of the host copies: in the upload
 * phase a task packs its source rows into pinned staging memory and enqueues
 * their host-to-device copy on the stream (copies of different tasks overlap
 * with each other and with the packing of later tasks); in the download
 * phase a task waits for its stripe's device-to-host copy and unpacks it into
 * `dst`.  The filter itself is one launch between the phases.  Images already
 * in pinned or device memory skip the packing.  Work runs on the calling
 * thread's default context (kleidicv_gpu_context_create on the current
 * device, first use).
 *
 * Errors: the reference's values and order; `mt.parallel == NULL` returns
 * KLEIDICV_ERROR_NULL_POINTER (the reference would call through it); a
 * scheduler that reports a failure makes the call return that failure.
 *
 * kleidicv_gpu_thread_pool_* is a ready-made scheduler: a persistent pool of
 * worker threads (the pattern of KleidiCV's examples/threading/main.cpp:52-86)
 * whose `parallel` function fulfils the contract:
 *   mt.parallel = kleidicv_gpu_thread_pool_parallel; mt.parallel_data = pool;
 */
#ifndef KLEIDICV_GPU_THREAD_H
#define KLEIDICV_GPU_THREAD_H

#include "kleidicv_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* The scheduler contract, identical to kleidicv_thread.h:56-97.  When the
 * reference header is included first its definitions are used. */
#ifndef KLEIDICV_THREAD_H
typedef kleidicv_error_t (*kleidicv_thread_callback)(unsigned begin, unsigned end, void *data);
typedef kleidicv_error_t (*kleidicv_thread_parallel)(kleidicv_thread_callback callback,
                                                     void *callback_data, void *parallel_data,
                                                     unsigned task_count);
typedef struct {
  kleidicv_thread_parallel parallel;
  void *parallel_data;
} kleidicv_thread_multithreading;
#endif

kleidicv_error_t kleidicv_gpu_thread_gaussian_blur_u8(
    const uint8_t *src, size_t src_stride, uint8_t *dst, size_t dst_stride, size_t width,
    size_t height, size_t channels, size_t kernel_width, size_t kernel_height, float sigma_x,
    float sigma_y, kleidicv_border_type_t border_type, kleidicv_thread_multithreading mt);

kleidicv_error_t kleidicv_gpu_thread_separable_filter_2d_u8(
    const uint8_t *src, size_t src_stride, uint8_t *dst, size_t dst_stride, size_t width,
    size_t height, size_t channels, const uint8_t *kernel_x, size_t kernel_width,
    const uint8_t *kernel_y, size_t kernel_height, kleidicv_border_type_t border_type,
    kleidicv_thread_multithreading mt);

kleidicv_error_t kleidicv_gpu_thread_separable_filter_2d_u16(
    const uint16_t *src, size_t src_stride, uint16_t *dst, size_t dst_stride, size_t width,
    size_t height, size_t channels, const uint16_t *kernel_x, size_t kernel_width,
    const uint16_t *kernel_y, size_t kernel_height, kleidicv_border_type_t border_type,
    kleidicv_thread_multithreading mt);

kleidicv_error_t kleidicv_gpu_thread_blur_and_downsample_u8(
    const uint8_t *src, size_t src_stride, size_t src_width, size_t src_height, uint8_t *dst,
    size_t dst_stride, size_t channels, kleidicv_border_type_t border_type,
    kleidicv_thread_multithreading mt);

kleidicv_error_t kleidicv_gpu_thread_sobel_3x3_horizontal_s16_u8(
    const uint8_t *src, size_t src_stride, int16_t *dst, size_t dst_stride, size_t width,
    size_t height, size_t channels, kleidicv_thread_multithreading mt);

kleidicv_error_t kleidicv_gpu_thread_sobel_3x3_vertical_s16_u8(
    const uint8_t *src, size_t src_stride, int16_t *dst, size_t dst_stride, size_t width,
    size_t height, size_t channels, kleidicv_thread_multithreading mt);

/* kleidicv_thread_median_blur_* (kleidicv_thread.h:496-524, u32/s32 from the
 * thread API's other element types). */
kleidicv_error_t kleidicv_gpu_thread_median_blur_s8(
    const int8_t *src, size_t src_stride, int8_t *dst, size_t dst_stride, size_t width, size_t height,
    size_t channels, size_t kernel_width, size_t kernel_height,
    kleidicv_border_type_t border_type, kleidicv_thread_multithreading mt);
kleidicv_error_t kleidicv_gpu_thread_median_blur_u8(
    const uint8_t *src, size_t src_stride, uint8_t *dst, size_t dst_stride, size_t width, size_t height,
    size_t channels, size_t kernel_width, size_t kernel_height,
    kleidicv_border_type_t border_type, kleidicv_thread_multithreading mt);
kleidicv_error_t kleidicv_gpu_thread_median_blur_u16(
    const uint16_t *src, size_t src_stride, uint16_t *dst, size_t dst_stride, size_t width, size_t height,
    size_t channels, size_t kernel_width, size_t kernel_height,
    kleidicv_border_type_t border_type, kleidicv_thread_multithreading mt);
kleidicv_error_t kleidicv_gpu_thread_median_blur_s16(
    const int16_t *src, size_t src_stride, int16_t *dst, size_t dst_stride, size_t width, size_t height,
    size_t channels, size_t kernel_width, size_t kernel_height,
    kleidicv_border_type_t border_type, kleidicv_thread_multithreading mt);
kleidicv_error_t kleidicv_gpu_thread_median_blur_u32(
    const uint32_t *src, size_t src_stride, uint32_t *dst, size_t dst_stride, size_t width, size_t height,
    size_t channels, size_t kernel_width, size_t kernel_height,
    kleidicv_border_type_t border_type, kleidicv_thread_multithreading mt);
kleidicv_error_t kleidicv_gpu_thread_median_blur_s32(
    const int32_t *src, size_t src_stride, int32_t *dst, size_t dst_stride, size_t width, size_t height,
    size_t channels, size_t kernel_width, size_t kernel_height,
    kleidicv_border_type_t border_type, kleidicv_thread_multithreading mt);
kleidicv_error_t kleidicv_gpu_thread_median_blur_f32(
    const float *src, size_t src_stride, float *dst, size_t dst_stride, size_t width, size_t height,
    size_t channels, size_t kernel_width, size_t kernel_height,
    kleidicv_border_type_t border_type, kleidicv_thread_multithreading mt);

/* ---- Asynchronous variant (no counterpart in the reference) -------------
 *
 * The same calls, returning once the work is enqueued instead of once `dst`
 * holds the result: the scheduler contract of kleidicv_thread.h:42-97 with a
 * completion callback instead of a blocking return.
 *
 *  - Validation is the synchronous call's, in its order; a call that fails it
 *    enqueues nothing, never calls `done` and sets *handle to NULL.
 *  - Before returning, the call runs the upload phase through `mt` (packing a
 *    pageable source into pinned staging) and enqueues the filter and the
 *    device-to-host copies on the calling thread's default context.
 *  - A library worker thread of that context then finishes the call: it runs
 *    the download phase through `mt` (unpacking into a pageable `dst`), frees
 *    the call's device memory, calls `done(status, user_data)` if `done` is
 *    not NULL, and marks the handle complete.  The scheduler's `parallel`
 *    must therefore accept calls from that thread.  Calls made from one
 *    thread complete in the order they were made.
 *  - `src` and `dst` must stay valid, and `src` unchanged, until completion.
 *  - With `handle` non-NULL the caller owns a handle: query it, wait on it and
 *    release it (release waits for completion).  With `handle` NULL the library
 *    releases everything itself after `done` returns.
 */
typedef struct kleidicv_gpu_async kleidicv_gpu_async_t;
typedef void (*kleidicv_gpu_async_callback)(kleidicv_error_t status, void *user_data);

kleidicv_error_t kleidicv_gpu_thread_gaussian_blur_u8_async(
    const uint8_t *src, size_t src_stride, uint8_t *dst, size_t dst_stride, size_t width,
    size_t height, size_t channels, size_t kernel_width, size_t kernel_height, float sigma_x,
    float sigma_y, kleidicv_border_type_t border_type, kleidicv_thread_multithreading mt,
    kleidicv_gpu_async_callback done, void *user_data, kleidicv_gpu_async_t **handle);

kleidicv_error_t kleidicv_gpu_thread_separable_filter_2d_u8_async(
    const uint8_t *src, size_t src_stride, uint8_t *dst, size_t dst_stride, size_t width,
    size_t height, size_t channels, const uint8_t *kernel_x, size_t kernel_width,
    const uint8_t *kernel_y, size_t kernel_height, kleidicv_border_type_t border_type,
    kleidicv_thread_multithreading mt, kleidicv_gpu_async_callback done, void *user_data,
    kleidicv_gpu_async_t **handle);

kleidicv_error_t kleidicv_gpu_thread_separable_filter_2d_u16_async(
    const uint16_t *src, size_t src_stride, uint16_t *dst, size_t dst_stride, size_t width,
    size_t height, size_t channels, const uint16_t *kernel_x, size_t kernel_width,
    const uint16_t *kernel_y, size_t kernel_height, kleidicv_border_type_t border_type,
    kleidicv_thread_multithreading mt, kleidicv_gpu_async_callback done, void *user_data,
    kleidicv_gpu_async_t **handle);

kleidicv_error_t kleidicv_gpu_thread_blur_and_downsample_u8_async(
    const uint8_t *src, size_t src_stride, size_t src_width, size_t src_height, uint8_t *dst,
    size_t dst_stride, size_t channels, kleidicv_border_type_t border_type,
    kleidicv_thread_multithreading mt, kleidicv_gpu_async_callback done, void *user_data,
    kleidicv_gpu_async_t **handle);

/* KLEIDICV_GPU_ERROR_NOT_READY while the call runs, then its final status. */
kleidicv_error_t kleidicv_gpu_async_query(const kleidicv_gpu_async_t *handle);
/* Blocks until the call completed; returns its final status. */
kleidicv_error_t kleidicv_gpu_async_wait(kleidicv_gpu_async_t *handle);
/* Waits for completion, then frees the handle. */
kleidicv_error_t kleidicv_gpu_async_release(kleidicv_gpu_async_t *handle);

/* A persistent worker pool implementing kleidicv_thread_parallel: `threads`
 * workers (0: the hardware concurrency) plus the calling thread take task
 * indices one at a time until all are done; the first failing callback's
 * error is returned.  One `parallel` call at a time per pool. */
typedef struct kleidicv_gpu_thread_pool kleidicv_gpu_thread_pool_t;
kleidicv_error_t kleidicv_gpu_thread_pool_create(kleidicv_gpu_thread_pool_t **pool,
                                                 unsigned threads);
kleidicv_error_t kleidicv_gpu_thread_pool_destroy(kleidicv_gpu_thread_pool_t *pool);
kleidicv_error_t kleidicv_gpu_thread_pool_parallel(kleidicv_thread_callback callback,
                                                   void *callback_data, void *parallel_data,
                                                   unsigned task_count);

#ifdef __cplusplus
}
#endif

#endif /* KLEIDICV_GPU_THREAD_H */
