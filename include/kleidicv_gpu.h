/*
 * kleidicv_gpu.h -- GB300 (sm_103a) drop-in for KleidiCV's separable-filter
 * hot path, exposed as a plain C ABI.
 *
 * Every drop-in entry point keeps the parameter list, the meaning of every
 * argument, the kleidicv_error_t values and the order in which errors are
 * detected of the KleidiCV function it replaces, and adds one trailing
 * `kleidicv_gpu_context_t *ctx` argument (the analogue of the trailing
 * `kleidicv_thread_multithreading mt` argument of KleidiCV's threaded API).
 *
 *  - src / dst are DEVICE pointers (cudaMalloc, a pool, or device-mapped
 *    memory); strides are in bytes.
 *  - Validation errors are returned synchronously, before any CUDA call.
 *  - Work is enqueued asynchronously on the context's stream; KLEIDICV_OK
 *    means "enqueued".  kleidicv_gpu_context_synchronize() waits and reports
 *    device-side failures.
 *  - There is no CPU fallback: a context can only be created on a CUDA device
 *    that runs sm_103a code, and entry points fail with
 *    KLEIDICV_GPU_ERROR_CUDA if the device work cannot be launched.
 *
 * Reference functions replaced (KleidiCV project paths):
 *  kleidicv_gpu_gaussian_blur_u8         kleidicv/include/kleidicv/kleidicv.h:2159-2163
 *                                        (kleidicv/src/filters/gaussian_blur_api.cpp:59-67)
 *  kleidicv_gpu_separable_filter_2d_u8   kleidicv/include/kleidicv/kleidicv.h:2091-2095
 *                                        (kleidicv/src/filters/separable_filter_2d_api.cpp:47-55)
 *  kleidicv_gpu_separable_filter_2d_u16  kleidicv/include/kleidicv/kleidicv.h:2103-2107
 *                                        (kleidicv/src/filters/separable_filter_2d_api.cpp:67-75)
 *  kleidicv_gpu_blur_and_downsample_u8   kleidicv/include/kleidicv/kleidicv.h:2215-2218
 *                                        (kleidicv/src/filters/blur_and_downsample_api.cpp:40-48)
 *  kleidicv_gpu_sobel_3x3_horizontal_s16_u8
 *                                        kleidicv/include/kleidicv/kleidicv.h:2050-2052
 *                                        (kleidicv/src/filters/sobel_api.cpp:37-43)
 *  kleidicv_gpu_sobel_3x3_vertical_s16_u8
 *                                        kleidicv/include/kleidicv/kleidicv.h:2006-2008
 *                                        (kleidicv/src/filters/sobel_api.cpp:53-58)
 *  kleidicv_gpu_<each of the six above>_sme
 *                                        kleidicv/include/kleidicv/kleidicv.h:2010,2054,2097,2109,2165,2220
 *  kleidicv_gpu_median_blur_{s8,u8,u16,s16,u32,s32,f32}
 *                                        kleidicv/include/kleidicv/kleidicv.h:2225-2302
 *                                        (kleidicv/src/filters/median_blur_api.cpp:42-242)
 * and, with the same argument lists, the threaded variants
 *  kleidicv_thread_{gaussian_blur_u8,separable_filter_2d_u8,
 *  separable_filter_2d_u16,blur_and_downsample_u8}
 *                                        kleidicv_thread/include/kleidicv_thread/kleidicv_thread.h:457-485
 * (the `mt` scheduler argument becomes the context).
 */
#ifndef KLEIDICV_GPU_H
#define KLEIDICV_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Error and border enums: identical values to kleidicv/include/kleidicv/ctypes.h:26-79.
 * When the reference header is included first its definitions are used. */
#ifndef KLEIDICV_CTYPES_H
typedef enum {
  KLEIDICV_OK = 0,
  KLEIDICV_ERROR_NOT_IMPLEMENTED,
  KLEIDICV_ERROR_NULL_POINTER,
  KLEIDICV_ERROR_RANGE,
  KLEIDICV_ERROR_ALLOCATION,
  KLEIDICV_ERROR_ALIGNMENT,
  KLEIDICV_ERROR_CONTEXT_MISMATCH,
} kleidicv_error_t;

typedef enum {
  KLEIDICV_BORDER_TYPE_CONSTANT,
  KLEIDICV_BORDER_TYPE_REPLICATE,
  KLEIDICV_BORDER_TYPE_REFLECT,
  KLEIDICV_BORDER_TYPE_WRAP,
  KLEIDICV_BORDER_TYPE_REVERSE,
  KLEIDICV_BORDER_TYPE_TRANSPARENT,
  KLEIDICV_BORDER_TYPE_NONE,
} kleidicv_border_type_t;
#endif

/* GPU-specific failures, returned as kleidicv_error_t values >= 0x100 so
 * that 0..6 keep the reference's meaning. */
#define KLEIDICV_GPU_ERROR_CUDA ((kleidicv_error_t)0x100)      /* a CUDA call failed */
#define KLEIDICV_GPU_ERROR_NO_DEVICE ((kleidicv_error_t)0x101) /* no usable sm_103 device */
#define KLEIDICV_GPU_ERROR_TIMEOUT ((kleidicv_error_t)0x102)   /* a device wait hit its limit */
#define KLEIDICV_GPU_ERROR_BUSY ((kleidicv_error_t)0x103)      /* serving queue full */
#define KLEIDICV_GPU_ERROR_NOT_READY ((kleidicv_error_t)0x104) /* asynchronous call still running */

/* KLEIDICV_MAX_IMAGE_PIXELS and KLEIDICV_MAXIMUM_CHANNEL_COUNT, kleidicv.h:103,110 */
#define KLEIDICV_GPU_MAX_IMAGE_PIXELS ((1ULL << 48) - 1)
#define KLEIDICV_GPU_MAXIMUM_CHANNEL_COUNT 4

/* ------------------------------------------------------------------------ */
/* Context: device, stream, device memory pool, error flag.                 */

typedef struct kleidicv_gpu_context kleidicv_gpu_context_t;

/* Creates a context on `device` that enqueues work on `stream` (a
 * cudaStream_t; NULL = the legacy default stream).  pool_limit_bytes caps the
 * context's device pool (0 = 40 GiB). */
kleidicv_error_t kleidicv_gpu_context_create(kleidicv_gpu_context_t **ctx,
                                             int device, void *stream,
                                             size_t pool_limit_bytes);
kleidicv_error_t kleidicv_gpu_context_destroy(kleidicv_gpu_context_t *ctx);
kleidicv_error_t kleidicv_gpu_context_set_stream(kleidicv_gpu_context_t *ctx,
                                                 void *stream);
void *kleidicv_gpu_context_get_stream(const kleidicv_gpu_context_t *ctx);
/* Waits for all work on the context's stream; reports CUDA errors and
 * device-side timeouts recorded since the last call. */
kleidicv_error_t kleidicv_gpu_context_synchronize(kleidicv_gpu_context_t *ctx);
/* Fault injection for tests: the next `count` pool allocations fail. */
void kleidicv_gpu_context_fail_next_allocations(kleidicv_gpu_context_t *ctx,
                                                int count);
/* Number of this library's kernels launched through the context so far. */
uint64_t kleidicv_gpu_context_launch_count(const kleidicv_gpu_context_t *ctx);
/* Tuning knob (no reference counterpart): forces the fused kernels' tile
 * shape for every later call on the context -- CTA threads (32..128, a
 * multiple of 32), output rows per tile (0: balanced over one wave), rows per
 * TMA stage and ring stages (0: the default depth; an explicit depth is
 * raised to the ring depth rule's minimum).
 * threads == 0 restores the committed autotune table / heuristic.  Used by
 * the package's autotuner to measure candidate shapes. */
kleidicv_error_t kleidicv_gpu_context_set_tile_shape(kleidicv_gpu_context_t *ctx, int threads,
                                                     int tile_rows, int stage_rows, int stages);

/* ------------------------------------------------------------------------ */
/* Drop-in entry points.                                                    */

kleidicv_error_t kleidicv_gpu_gaussian_blur_u8(
    const uint8_t *src, size_t src_stride, uint8_t *dst, size_t dst_stride,
    size_t width, size_t height, size_t channels, size_t kernel_width,
    size_t kernel_height, float sigma_x, float sigma_y,
    kleidicv_border_type_t border_type, kleidicv_gpu_context_t *ctx);

kleidicv_error_t kleidicv_gpu_separable_filter_2d_u8(
    const uint8_t *src, size_t src_stride, uint8_t *dst, size_t dst_stride,
    size_t width, size_t height, size_t channels, const uint8_t *kernel_x,
    size_t kernel_width, const uint8_t *kernel_y, size_t kernel_height,
    kleidicv_border_type_t border_type, kleidicv_gpu_context_t *ctx);

kleidicv_error_t kleidicv_gpu_separable_filter_2d_u16(
    const uint16_t *src, size_t src_stride, uint16_t *dst, size_t dst_stride,
    size_t width, size_t height, size_t channels, const uint16_t *kernel_x,
    size_t kernel_width, const uint16_t *kernel_y, size_t kernel_height,
    kleidicv_border_type_t border_type, kleidicv_gpu_context_t *ctx);

kleidicv_error_t kleidicv_gpu_blur_and_downsample_u8(
    const uint8_t *src, size_t src_stride, size_t src_width, size_t src_height,
    uint8_t *dst, size_t dst_stride, size_t channels,
    kleidicv_border_type_t border_type, kleidicv_gpu_context_t *ctx);

/* 3x3 Sobel derivatives, u8 -> s16, REPLICATE border (the reference's only
 * one; there is no border argument).  horizontal = d/dx: [1 2 1]^T x
 * [-1 0 1]; vertical = d/dy: [-1 0 1]^T x [1 2 1].  width, height >= 2, else
 * NOT_IMPLEMENTED; dst_stride must be even when height > 1 (ALIGNMENT). */
kleidicv_error_t kleidicv_gpu_sobel_3x3_horizontal_s16_u8(
    const uint8_t *src, size_t src_stride, int16_t *dst, size_t dst_stride,
    size_t width, size_t height, size_t channels, kleidicv_gpu_context_t *ctx);

kleidicv_error_t kleidicv_gpu_sobel_3x3_vertical_s16_u8(
    const uint8_t *src, size_t src_stride, int16_t *dst, size_t dst_stride,
    size_t width, size_t height, size_t channels, kleidicv_gpu_context_t *ctx);

/* The `_sme` twins (kleidicv.h:2010, 2054, 2097, 2109, 2165, 2220): in KleidiCV
 * the suffix selects the CPU backend and changes neither semantics nor the
 * parameter contract (kleidicv.h:23-35); here each twin is the same call as
 * its base entry. */
kleidicv_error_t kleidicv_gpu_gaussian_blur_u8_sme(
    const uint8_t *src, size_t src_stride, uint8_t *dst, size_t dst_stride,
    size_t width, size_t height, size_t channels, size_t kernel_width,
    size_t kernel_height, float sigma_x, float sigma_y,
    kleidicv_border_type_t border_type, kleidicv_gpu_context_t *ctx);
kleidicv_error_t kleidicv_gpu_separable_filter_2d_u8_sme(
    const uint8_t *src, size_t src_stride, uint8_t *dst, size_t dst_stride,
    size_t width, size_t height, size_t channels, const uint8_t *kernel_x,
    size_t kernel_width, const uint8_t *kernel_y, size_t kernel_height,
    kleidicv_border_type_t border_type, kleidicv_gpu_context_t *ctx);
kleidicv_error_t kleidicv_gpu_separable_filter_2d_u16_sme(
    const uint16_t *src, size_t src_stride, uint16_t *dst, size_t dst_stride,
    size_t width, size_t height, size_t channels, const uint16_t *kernel_x,
    size_t kernel_width, const uint16_t *kernel_y, size_t kernel_height,
    kleidicv_border_type_t border_type, kleidicv_gpu_context_t *ctx);
kleidicv_error_t kleidicv_gpu_blur_and_downsample_u8_sme(
    const uint8_t *src, size_t src_stride, size_t src_width, size_t src_height,
    uint8_t *dst, size_t dst_stride, size_t channels,
    kleidicv_border_type_t border_type, kleidicv_gpu_context_t *ctx);
kleidicv_error_t kleidicv_gpu_sobel_3x3_horizontal_s16_u8_sme(
    const uint8_t *src, size_t src_stride, int16_t *dst, size_t dst_stride,
    size_t width, size_t height, size_t channels, kleidicv_gpu_context_t *ctx);
kleidicv_error_t kleidicv_gpu_sobel_3x3_vertical_s16_u8_sme(
    const uint8_t *src, size_t src_stride, int16_t *dst, size_t dst_stride,
    size_t width, size_t height, size_t channels, kleidicv_gpu_context_t *ctx);

/* Median blur of the K x K window (kleidicv.h:2225-2302; validation
 * kleidicv/include/kleidicv/filters/median_blur.h:148-193): K odd, 3..7 for
 * every type, 3..255 for u8; REPLICATE, REFLECT, WRAP or REVERSE; width and
 * height >= K - 1; src != dst.  The median of the window is unique, so the
 * results equal the reference's sorting networks and histograms (f32: for
 * inputs without NaN; -0.0 orders below +0.0). */
kleidicv_error_t kleidicv_gpu_median_blur_s8(
    const int8_t *src, size_t src_stride, int8_t *dst, size_t dst_stride, size_t width,
    size_t height, size_t channels, size_t kernel_width, size_t kernel_height,
    kleidicv_border_type_t border_type, kleidicv_gpu_context_t *ctx);
kleidicv_error_t kleidicv_gpu_median_blur_u8(
    const uint8_t *src, size_t src_stride, uint8_t *dst, size_t dst_stride, size_t width,
    size_t height, size_t channels, size_t kernel_width, size_t kernel_height,
    kleidicv_border_type_t border_type, kleidicv_gpu_context_t *ctx);
kleidicv_error_t kleidicv_gpu_median_blur_u16(
    const uint16_t *src, size_t src_stride, uint16_t *dst, size_t dst_stride, size_t width,
    size_t height, size_t channels, size_t kernel_width, size_t kernel_height,
    kleidicv_border_type_t border_type, kleidicv_gpu_context_t *ctx);
kleidicv_error_t kleidicv_gpu_median_blur_s16(
    const int16_t *src, size_t src_stride, int16_t *dst, size_t dst_stride, size_t width,
    size_t height, size_t channels, size_t kernel_width, size_t kernel_height,
    kleidicv_border_type_t border_type, kleidicv_gpu_context_t *ctx);
kleidicv_error_t kleidicv_gpu_median_blur_u32(
    const uint32_t *src, size_t src_stride, uint32_t *dst, size_t dst_stride, size_t width,
    size_t height, size_t channels, size_t kernel_width, size_t kernel_height,
    kleidicv_border_type_t border_type, kleidicv_gpu_context_t *ctx);
kleidicv_error_t kleidicv_gpu_median_blur_s32(
    const int32_t *src, size_t src_stride, int32_t *dst, size_t dst_stride, size_t width,
    size_t height, size_t channels, size_t kernel_width, size_t kernel_height,
    kleidicv_border_type_t border_type, kleidicv_gpu_context_t *ctx);
kleidicv_error_t kleidicv_gpu_median_blur_f32(
    const float *src, size_t src_stride, float *dst, size_t dst_stride, size_t width,
    size_t height, size_t channels, size_t kernel_width, size_t kernel_height,
    kleidicv_border_type_t border_type, kleidicv_gpu_context_t *ctx);

/* ------------------------------------------------------------------------ */
/* Extensions (no reference counterpart; semantics defined by this library,
 * "parity unpinned"):
 *  - KLEIDICV_BORDER_TYPE_CONSTANT with an explicit border_value: the image
 *    is treated as padded with border_value on every side (the definition
 *    the reference's own test framework uses, test/framework/border.cpp:369-415);
 *  - the s16 separable filter, whose declaration exists in the reference
 *    (kleidicv/include/kleidicv/filters/separable_filter_2d.h:34-43) without
 *    a definition: 32-bit vertical accumulation with saturating adds in tap
 *    order, 64-bit horizontal accumulation, saturation to s16.
 * For the four fixed border types the _ex functions return exactly what the
 * drop-in functions return.  Kernel taps (kernel_x / kernel_y) are HOST
 * pointers in every separable entry point, as in the reference. */

kleidicv_error_t kleidicv_gpu_gaussian_blur_u8_ex(
    const uint8_t *src, size_t src_stride, uint8_t *dst, size_t dst_stride,
    size_t width, size_t height, size_t channels, size_t kernel_width,
    size_t kernel_height, float sigma_x, float sigma_y,
    kleidicv_border_type_t border_type, uint8_t border_value,
    kleidicv_gpu_context_t *ctx);

kleidicv_error_t kleidicv_gpu_separable_filter_2d_u8_ex(
    const uint8_t *src, size_t src_stride, uint8_t *dst, size_t dst_stride,
    size_t width, size_t height, size_t channels, const uint8_t *kernel_x,
    size_t kernel_width, const uint8_t *kernel_y, size_t kernel_height,
    kleidicv_border_type_t border_type, uint8_t border_value,
    kleidicv_gpu_context_t *ctx);

kleidicv_error_t kleidicv_gpu_separable_filter_2d_u16_ex(
    const uint16_t *src, size_t src_stride, uint16_t *dst, size_t dst_stride,
    size_t width, size_t height, size_t channels, const uint16_t *kernel_x,
    size_t kernel_width, const uint16_t *kernel_y, size_t kernel_height,
    kleidicv_border_type_t border_type, uint16_t border_value,
    kleidicv_gpu_context_t *ctx);

kleidicv_error_t kleidicv_gpu_separable_filter_2d_s16_ex(
    const int16_t *src, size_t src_stride, int16_t *dst, size_t dst_stride,
    size_t width, size_t height, size_t channels, const int16_t *kernel_x,
    size_t kernel_width, const int16_t *kernel_y, size_t kernel_height,
    kleidicv_border_type_t border_type, int16_t border_value,
    kleidicv_gpu_context_t *ctx);

kleidicv_error_t kleidicv_gpu_blur_and_downsample_u8_ex(
    const uint8_t *src, size_t src_stride, size_t src_width, size_t src_height,
    uint8_t *dst, size_t dst_stride, size_t channels,
    kleidicv_border_type_t border_type, uint8_t border_value,
    kleidicv_gpu_context_t *ctx);

/* Image pyramid: `levels` successive blur_and_downsample_u8 steps.  Level l
 * (1-based) has size ((w_{l-1}+1)/2, (h_{l-1}+1)/2) and is written to
 * dst[l-1] with stride dst_strides[l-1].  The caller of the reference builds
 * the same pyramid by calling kleidicv_blur_and_downsample_u8 once per level
 * (kleidicv/include/kleidicv/analysis/build_optical_flow_pyr_lk_pyramid.h:359-380).
 * Validation is per level, in level order, with the drop-in's rules. */
kleidicv_error_t kleidicv_gpu_build_pyramid_u8(
    const uint8_t *src, size_t src_stride, size_t src_width, size_t src_height,
    size_t channels, size_t levels, uint8_t *const *dst,
    const size_t *dst_strides, kleidicv_border_type_t border_type,
    kleidicv_gpu_context_t *ctx);

/* ------------------------------------------------------------------------ */
/* Lucas-Kanade pyramid: the image and Scharr pyramids that
 * kleidicv_build_optical_flow_pyr_lk_pyramid builds
 * (kleidicv/include/kleidicv/kleidicv.h:361-364,
 * kleidicv/src/analysis/build_optical_flow_pyr_lk_pyramid_api.cpp:13-48), in
 * device memory.  Same arguments, validation order and level-count rule;
 * level l >= 1 is blur_and_downsample (REVERSE) of level l-1.  Every level
 * holds its image with a reflect-101 border of (window_width, window_height)
 * pixels and the interleaved (dx, dy) Scharr derivatives (s16, 2 x channels
 * per pixel) with a zero halo of the same size.  kleidicv_gpu_lk_pyramid_level
 * returns DEVICE pointers to a level's interiors (the reference keeps its
 * layout opaque; this accessor is the GPU handle's way to reach the data). */
typedef struct kleidicv_gpu_lk_pyramid kleidicv_gpu_lk_pyramid_t;

kleidicv_error_t kleidicv_gpu_build_optical_flow_pyr_lk_pyramid(
    kleidicv_gpu_lk_pyramid_t **pyramid, const uint8_t *src, size_t src_stride, size_t width,
    size_t height, size_t channels, size_t level_count, size_t window_width,
    size_t window_height, kleidicv_gpu_context_t *ctx);
/* kleidicv_optical_flow_pyr_lk_pyramid_release (kleidicv.h:377-378). */
kleidicv_error_t kleidicv_gpu_optical_flow_pyr_lk_pyramid_release(
    kleidicv_gpu_lk_pyramid_t *pyramid);
size_t kleidicv_gpu_lk_pyramid_level_count(const kleidicv_gpu_lk_pyramid_t *pyramid);
kleidicv_error_t kleidicv_gpu_lk_pyramid_level(const kleidicv_gpu_lk_pyramid_t *pyramid,
                                               size_t level, size_t *width, size_t *height,
                                               const uint8_t **image, size_t *image_stride,
                                               const int16_t **scharr, size_t *scharr_stride,
                                               size_t *border_width, size_t *border_height);

/* ------------------------------------------------------------------------ */
/* Batched execution: many independent filter requests of uneven sizes run
 * through one persistent kernel that walks a device-side tile work-list.  A
 * plan is built once (validation, tile list, tensor maps, tile shapes from
 * the autotune table) and can be launched repeatedly; plan launches may be
 * captured into a CUDA graph. */

typedef enum {
  KLEIDICV_GPU_OP_GAUSSIAN_BLUR_U8 = 0,
  KLEIDICV_GPU_OP_SEPARABLE_FILTER_2D_U8 = 1,
  KLEIDICV_GPU_OP_SEPARABLE_FILTER_2D_U16 = 2,
  KLEIDICV_GPU_OP_SEPARABLE_FILTER_2D_S16 = 3,
  KLEIDICV_GPU_OP_BLUR_AND_DOWNSAMPLE_U8 = 4,
} kleidicv_gpu_op_t;

typedef struct {
  kleidicv_gpu_op_t op;
  const void *src; /* device */
  size_t src_stride;
  void *dst; /* device */
  size_t dst_stride;
  size_t width, height, channels; /* source size, as in the drop-in calls */
  size_t kernel_width, kernel_height;
  float sigma_x, sigma_y;     /* gaussian */
  int32_t kernel_x[5];        /* separable taps (value range of the op's type) */
  int32_t kernel_y[5];
  kleidicv_border_type_t border_type;
  int32_t border_value;       /* CONSTANT border only (extension) */
  int32_t allow_extensions;   /* 0: drop-in validation; 1: _ex validation */
} kleidicv_gpu_request_t;

typedef struct kleidicv_gpu_batch_plan kleidicv_gpu_batch_plan_t;

/* Validates every request (statuses[i] receives each request's
 * kleidicv_error_t, exactly what the corresponding single call would
 * return) and builds a plan for the valid ones.  Returns KLEIDICV_OK if the
 * plan was built (even if some requests were rejected). */
kleidicv_error_t kleidicv_gpu_batch_plan_create(
    const kleidicv_gpu_request_t *requests, size_t count,
    kleidicv_error_t *statuses, kleidicv_gpu_batch_plan_t **plan,
    kleidicv_gpu_context_t *ctx);
/* Enqueues the plan: one persistent-kernel launch (plus its work-counter
 * reset), on the context's stream.  use_graph != 0 replays a CUDA graph
 * captured on first use. */
kleidicv_error_t kleidicv_gpu_batch_plan_launch(kleidicv_gpu_batch_plan_t *plan,
                                                int use_graph,
                                                kleidicv_gpu_context_t *ctx);
kleidicv_error_t kleidicv_gpu_batch_plan_destroy(kleidicv_gpu_batch_plan_t *plan);
/* Number of tiles in the plan's work-list. */
size_t kleidicv_gpu_batch_plan_tile_count(const kleidicv_gpu_batch_plan_t *plan);

/* One-shot convenience: plan + launch + destroy (destroy is deferred until
 * the launch has completed). */
kleidicv_error_t kleidicv_gpu_batch_submit(const kleidicv_gpu_request_t *requests,
                                           size_t count,
                                           kleidicv_error_t *statuses,
                                           kleidicv_gpu_context_t *ctx);

/* Many image pyramids in one launch per channel count (no reference
 * counterpart: the reference builds every pyramid level by level).  Each
 * entry is validated like kleidicv_gpu_build_pyramid_u8 (statuses[i] is its
 * result, statuses may be NULL); valid entries are computed, level l of every
 * image before level l + 1 of any.  Returns the first failing entry's status
 * (nothing is launched then) or a CUDA failure. */
typedef struct {
  const uint8_t *src;
  size_t src_stride, src_width, src_height, channels, levels;
  uint8_t *const *dst;
  const size_t *dst_strides;
  kleidicv_border_type_t border_type;
} kleidicv_gpu_pyramid_t;
kleidicv_error_t kleidicv_gpu_build_pyramids_u8(const kleidicv_gpu_pyramid_t *pyramids,
                                                size_t count, kleidicv_error_t *statuses,
                                                kleidicv_gpu_context_t *ctx);

/* ------------------------------------------------------------------------ */
/* Serving loop: requests arrive asynchronously, images stay resident in a
 * capped device pool, requests are admitted by free bytes and by free
 * in-flight slots, and every scheduling round launches one persistent batch
 * for everything admitted since the previous round while earlier batches are
 * still running (continuous batching over several streams). */

typedef struct kleidicv_gpu_server kleidicv_gpu_server_t;

typedef struct {
  size_t pool_limit_bytes;    /* device pool cap (0 = 40 GiB) */
  int max_inflight_batches;   /* batches allowed on the GPU at once (0 = 3) */
  int max_batch_requests;     /* requests per batch (0 = 512) */
  int max_queue;              /* pending requests before BUSY (0 = 65536) */
  size_t max_batch_bytes;     /* work budget of one batch: the requests' image
                                 bytes read plus written; a batch takes the
                                 oldest requests until the budget is reached,
                                 at least one (0 = no budget) */
} kleidicv_gpu_server_config_t;

typedef struct {
  uint64_t id;
  kleidicv_error_t status;
  double arrival_s, admitted_s, completed_s; /* server clock, seconds */
} kleidicv_gpu_completion_t;

kleidicv_error_t kleidicv_gpu_server_create(const kleidicv_gpu_server_config_t *config,
                                            int device, kleidicv_gpu_server_t **server);
kleidicv_error_t kleidicv_gpu_server_destroy(kleidicv_gpu_server_t *server);
/* Allocates `bytes` of device memory from the server's pool (for request
 * images).  Returns NULL when the pool cap would be exceeded. */
void *kleidicv_gpu_server_alloc(kleidicv_gpu_server_t *server, size_t bytes);
void kleidicv_gpu_server_free(kleidicv_gpu_server_t *server, void *ptr);
/* Queues a request; returns its id in *id.  The request's src/dst must stay
 * valid until its completion is reported. */
kleidicv_error_t kleidicv_gpu_server_submit(kleidicv_gpu_server_t *server,
                                            const kleidicv_gpu_request_t *request,
                                            uint64_t *id);
/* Copies up to `capacity` completions (in completion order) into `out`;
 * waits up to timeout_ms for at least one.  Returns the number copied. */
size_t kleidicv_gpu_server_poll(kleidicv_gpu_server_t *server,
                                kleidicv_gpu_completion_t *out, size_t capacity,
                                int timeout_ms);
/* Seconds on the server clock (the clock the completion times use). */
double kleidicv_gpu_server_now(const kleidicv_gpu_server_t *server);
/* Waits until every submitted request has completed. */
kleidicv_error_t kleidicv_gpu_server_drain(kleidicv_gpu_server_t *server);

/* ------------------------------------------------------------------------ */
/* Allocation-free arbitrary-size Gaussian.  No counterpart in the reference:
 * kleidicv_gaussian_blur_u8 (kleidicv.h:2159-2163) allocates its workspace
 * with malloc on every call (kleidicv/include/kleidicv/workspace/separable.h:82-100).
 *
 * For callers that must not allocate device memory on the call path:
 *  - a process that reserved its whole device budget at start-up;
 *  - a latency-critical loop, where an allocation (or the device-wide
 *    synchronisation a cudaFree can imply) is not acceptable;
 *  - a caller that holds no kleidicv_gpu_context_t (creating one allocates
 *    its error word).
 * kleidicv_gpu_gaussian_blur_u8 takes the intermediate image of its two-pass
 * arbitrary-size kernel from the context's pool on every call.  This entry
 * takes it from a fixed buffer that is part of the library's device image
 * (KLEIDICV_GPU_NOALLOC_SCRATCH_BYTES on every device that runs it), and it
 * calls no allocating routine.
 *
 *  - Arguments, validation order and results are those of
 *    kleidicv_gpu_gaussian_blur_u8, with a cudaStream_t in place of the
 *    context.
 *  - It serves the requests that entry computes with the two-pass kernel,
 *    and those whose kernel is a plain copy.  The two-pass requests are odd
 *    sizes 11..255 other than 15 and 21 with a REPLICATE border (the
 *    reference's arbitrary-size path), and generated kernels whose weights
 *    do not sum to 256.
 *  - Requests that the fused kernels compute return
 *    KLEIDICV_ERROR_NOT_IMPLEMENTED.  They need no scratch: call
 *    kleidicv_gpu_gaussian_blur_u8 with a context created at set-up.
 *  - Limit: ceil16(width * channels) * height must not exceed
 *    KLEIDICV_GPU_NOALLOC_SCRATCH_BYTES, otherwise KLEIDICV_ERROR_RANGE.
 *    This is checked after the drop-in validation.
 *  - There is one buffer per device.  Calls whose device work can overlap
 *    race on it and give wrong results: calls on different streams, or from
 *    several host threads on different streams.  Issue them on one stream,
 *    or order the streams with events.
 *  - Nothing has to start at zero: the first kernel writes every scratch
 *    byte that the second one reads.
 *  - The first call on each device (with that device current) does a
 *    one-time set-up.  It resolves the buffer's address
 *    (cudaGetSymbolAddress) and loads the two kernels, which makes CUDA load
 *    the library's device code on that device.  Make that first call before
 *    any stream capture. */
#define KLEIDICV_GPU_NOALLOC_SCRATCH_BYTES ((size_t)32 << 20)

kleidicv_error_t kleidicv_gpu_gaussian_blur_u8_noalloc(
    const uint8_t *src, size_t src_stride, uint8_t *dst, size_t dst_stride,
    size_t width, size_t height, size_t channels, size_t kernel_width,
    size_t kernel_height, float sigma_x, float sigma_y,
    kleidicv_border_type_t border_type, void *stream);

/* ------------------------------------------------------------------------ */
/* Failure-path self-test (no reference counterpart): enqueues a kernel whose
 * bounded wait on an mbarrier that nothing arrives at gives up after
 * limit_ns (1 ns .. 1 s), as a fused kernel does when its copies never land.
 * kleidicv_gpu_context_synchronize then reports KLEIDICV_GPU_ERROR_TIMEOUT
 * once, and the context stays usable. */
kleidicv_error_t kleidicv_gpu_selftest_bounded_wait(kleidicv_gpu_context_t *ctx,
                                                    uint64_t limit_ns);

/* ------------------------------------------------------------------------ */
/* Introspection (used by tests): the Gaussian half kernel this library
 * derives from (kernel_size, sigma), with the reference's generator
 * (kleidicv/include/kleidicv/filters/sigma.h:27-79).  Returns 1 and fills
 * kernel_size/2+1 weights, or 0 for the "copy" case. */
int kleidicv_gpu_gaussian_half_kernel(size_t kernel_size, float sigma,
                                      uint8_t *half_kernel);

#ifdef __cplusplus
}
#endif

#endif /* KLEIDICV_GPU_H */
