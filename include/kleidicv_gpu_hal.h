/*
 * kleidicv_gpu_hal.h -- OpenCV custom-HAL shim over the GB300 library.
 *
 * Routes cv::GaussianBlur, cv::sepFilter2D, cv::pyrDown and cv::Sobel to the
 * kleidicv_gpu_* entry points, with the acceptance rules, border mapping and
 * error mapping of KleidiCV's own OpenCV HAL adapter
 * (adapters/opencv/kleidicv_hal.cpp):
 *
 *  kleidicv_gpu_hal_separable_filter_2d      kleidicv_hal.cpp:453-549
 *  kleidicv_gpu_hal_gaussian_blur_binomial   kleidicv_hal.cpp:551-584
 *  kleidicv_gpu_hal_gaussian_blur            kleidicv_hal.cpp:586-621
 *  kleidicv_gpu_hal_pyrdown                  kleidicv_hal.cpp:1562-1592
 *  kleidicv_gpu_hal_sobel                    kleidicv_hal.cpp:821-879
 *  border mapping (from_opencv)              kleidicv_hal.cpp:405-435
 *  error mapping (convert_error)             kleidicv_hal.cpp:78-91
 *
 * The parameter lists are the OpenCV HAL hooks' (cv_hal_sepFilter_stateless,
 * cv_hal_gaussianBlurBinomial, cv_hal_gaussianBlur, cv_hal_pyrdown,
 * cv_hal_sobel).  OpenCV passes HOST pointers (cv::Mat data): the shim then
 * stages the image through device memory on the calling thread's default
 * context (upload, filter, download).  Device pointers (CUDA allocations,
 * managed memory) are filtered in place.  Every call is synchronous, as the
 * HAL contract requires.
 *
 * Return values: CV_HAL_ERROR_OK (0); CV_HAL_ERROR_NOT_IMPLEMENTED (1) when
 * the call falls outside what the reference adapter accepts (OpenCV then runs
 * its own code); CV_HAL_ERROR_UNKNOWN (-1) for every other failure, including
 * "no sm_103 device": OpenCV raises an error instead of silently computing
 * elsewhere.
 *
 * Wiring into an OpenCV build: include this header from the custom HAL header
 * after opencv2/core/hal/interface.h and define KLEIDICV_GPU_HAL_REPLACE; the
 * block at the end then points the five hooks at the shim, each falling back
 * to the previously defined hook when the shim answers NOT_IMPLEMENTED.
 */
#ifndef KLEIDICV_GPU_HAL_H
#define KLEIDICV_GPU_HAL_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

int kleidicv_gpu_hal_separable_filter_2d(
    const unsigned char *src_data, size_t src_step, int src_type, unsigned char *dst_data,
    size_t dst_step, int dst_type, int width, int height, int full_width, int full_height,
    int offset_x, int offset_y, const unsigned char *kernelx_data, int kernelx_len,
    const unsigned char *kernely_data, int kernely_len, int kernel_type, int anchor_x,
    int anchor_y, double delta, int border_type);

int kleidicv_gpu_hal_gaussian_blur_binomial(
    const unsigned char *src_data, size_t src_step, unsigned char *dst_data, size_t dst_step,
    int width, int height, int depth, int cn, size_t margin_left, size_t margin_top,
    size_t margin_right, size_t margin_bottom, size_t kernel_size, int border_type);

int kleidicv_gpu_hal_gaussian_blur(
    const unsigned char *src_data, size_t src_step, unsigned char *dst_data, size_t dst_step,
    int width, int height, int depth, int cn, size_t margin_left, size_t margin_top,
    size_t margin_right, size_t margin_bottom, size_t kernel_width, size_t kernel_height,
    double sigma_x, double sigma_y, int border_type);

int kleidicv_gpu_hal_pyrdown(const unsigned char *src_data, size_t src_step, int src_width,
                             int src_height, unsigned char *dst_data, size_t dst_step,
                             int dst_width, int dst_height, int depth, int cn, int border_type);

int kleidicv_gpu_hal_sobel(const unsigned char *src_data, size_t src_step,
                           unsigned char *dst_data, size_t dst_step, int width, int height,
                           int src_depth, int dst_depth, int cn, int margin_left,
                           int margin_top, int margin_right, int margin_bottom, int dx, int dy,
                           int ksize, double scale, double delta, int border_type);

#ifdef __cplusplus
}
#endif

#if defined(KLEIDICV_GPU_HAL_REPLACE) && defined(OPENCV_HAL_INTERFACE_H)
/* Custom-HAL wiring (compiled inside OpenCV's build only). */
static inline int kleidicv_gpu_sepFilter_with_fallback(
    const uchar *src_data, size_t src_step, int src_type, uchar *dst_data, size_t dst_step,
    int dst_type, int width, int height, int full_width, int full_height, int offset_x,
    int offset_y, uchar *kernelx_data, int kernelx_len, uchar *kernely_data, int kernely_len,
    int kernel_type, int anchor_x, int anchor_y, double delta, int border_type) {
  int r = kleidicv_gpu_hal_separable_filter_2d(
      src_data, src_step, src_type, dst_data, dst_step, dst_type, width, height, full_width,
      full_height, offset_x, offset_y, kernelx_data, kernelx_len, kernely_data, kernely_len,
      kernel_type, anchor_x, anchor_y, delta, border_type);
  return r != CV_HAL_ERROR_NOT_IMPLEMENTED
             ? r
             : cv_hal_sepFilter_stateless(src_data, src_step, src_type, dst_data, dst_step,
                                          dst_type, width, height, full_width, full_height,
                                          offset_x, offset_y, kernelx_data, kernelx_len,
                                          kernely_data, kernely_len, kernel_type, anchor_x,
                                          anchor_y, delta, border_type);
}
#undef cv_hal_sepFilter_stateless
#define cv_hal_sepFilter_stateless kleidicv_gpu_sepFilter_with_fallback

static inline int kleidicv_gpu_gaussianBlurBinomial_with_fallback(
    const uchar *src_data, size_t src_step, uchar *dst_data, size_t dst_step, int width,
    int height, int depth, int cn, size_t margin_left, size_t margin_top, size_t margin_right,
    size_t margin_bottom, size_t ksize, int border_type) {
  int r = kleidicv_gpu_hal_gaussian_blur_binomial(src_data, src_step, dst_data, dst_step, width,
                                                  height, depth, cn, margin_left, margin_top,
                                                  margin_right, margin_bottom, ksize, border_type);
  return r != CV_HAL_ERROR_NOT_IMPLEMENTED
             ? r
             : cv_hal_gaussianBlurBinomial(src_data, src_step, dst_data, dst_step, width, height,
                                           depth, cn, margin_left, margin_top, margin_right,
                                           margin_bottom, ksize, border_type);
}
#undef cv_hal_gaussianBlurBinomial
#define cv_hal_gaussianBlurBinomial kleidicv_gpu_gaussianBlurBinomial_with_fallback

static inline int kleidicv_gpu_gaussianBlur_with_fallback(
    const uchar *src_data, size_t src_step, uchar *dst_data, size_t dst_step, int width,
    int height, int depth, int cn, size_t margin_left, size_t margin_top, size_t margin_right,
    size_t margin_bottom, size_t ksize_width, size_t ksize_height, double sigma_x,
    double sigma_y, int border_type) {
  int r = kleidicv_gpu_hal_gaussian_blur(src_data, src_step, dst_data, dst_step, width, height,
                                         depth, cn, margin_left, margin_top, margin_right,
                                         margin_bottom, ksize_width, ksize_height, sigma_x,
                                         sigma_y, border_type);
  return r != CV_HAL_ERROR_NOT_IMPLEMENTED
             ? r
             : cv_hal_gaussianBlur(src_data, src_step, dst_data, dst_step, width, height, depth,
                                   cn, margin_left, margin_top, margin_right, margin_bottom,
                                   ksize_width, ksize_height, sigma_x, sigma_y, border_type);
}
#undef cv_hal_gaussianBlur
#define cv_hal_gaussianBlur kleidicv_gpu_gaussianBlur_with_fallback

static inline int kleidicv_gpu_pyrdown_with_fallback(const uchar *src_data, size_t src_step,
                                                     int src_width, int src_height,
                                                     uchar *dst_data, size_t dst_step,
                                                     int dst_width, int dst_height, int depth,
                                                     int cn, int border_type) {
  int r = kleidicv_gpu_hal_pyrdown(src_data, src_step, src_width, src_height, dst_data, dst_step,
                                   dst_width, dst_height, depth, cn, border_type);
  return r != CV_HAL_ERROR_NOT_IMPLEMENTED
             ? r
             : cv_hal_pyrdown(src_data, src_step, src_width, src_height, dst_data, dst_step,
                              dst_width, dst_height, depth, cn, border_type);
}
#undef cv_hal_pyrdown
#define cv_hal_pyrdown kleidicv_gpu_pyrdown_with_fallback

static inline int kleidicv_gpu_sobel_with_fallback(
    const uchar *src_data, size_t src_step, uchar *dst_data, size_t dst_step, int width,
    int height, int src_depth, int dst_depth, int cn, int margin_left, int margin_top,
    int margin_right, int margin_bottom, int dx, int dy, int ksize, double scale, double delta,
    int border_type) {
  int r = kleidicv_gpu_hal_sobel(src_data, src_step, dst_data, dst_step, width, height, src_depth,
                                 dst_depth, cn, margin_left, margin_top, margin_right,
                                 margin_bottom, dx, dy, ksize, scale, delta, border_type);
  return r != CV_HAL_ERROR_NOT_IMPLEMENTED
             ? r
             : cv_hal_sobel(src_data, src_step, dst_data, dst_step, width, height, src_depth,
                            dst_depth, cn, margin_left, margin_top, margin_right, margin_bottom,
                            dx, dy, ksize, scale, delta, border_type);
}
#undef cv_hal_sobel
#define cv_hal_sobel kleidicv_gpu_sobel_with_fallback
#endif /* KLEIDICV_GPU_HAL_REPLACE && OPENCV_HAL_INTERFACE_H */

#endif /* KLEIDICV_GPU_HAL_H */
