// The `_sme` twins of the drop-in entry points.
//
// KleidiCV declares a `_sme` variant beside each entry of this path
// (kleidicv/include/kleidicv/kleidicv.h:2010, 2054, 2097, 2109, 2165, 2220).
// The suffix selects the CPU backend (SME/SME2 when present, Neon or SVE2
// otherwise) and changes neither the semantics nor the parameter contract
// (kleidicv.h:23-35).  On the GPU there is one backend, so each twin is the
// same call: a caller that links the `_sme` names swaps them like the others.
#include "host.h"

extern "C" {

kleidicv_error_t kleidicv_gpu_gaussian_blur_u8_sme(const uint8_t *src, size_t src_stride, uint8_t *dst,
                                                   size_t dst_stride, size_t width, size_t height,
                                                   size_t channels, size_t kernel_width, size_t kernel_height,
                                                   float sigma_x, float sigma_y,
                                                   kleidicv_border_type_t border_type,
                                                   kleidicv_gpu_context_t *ctx) {
  return kleidicv_gpu_gaussian_blur_u8(src, src_stride, dst, dst_stride, width, height, channels, kernel_width,
                                       kernel_height, sigma_x, sigma_y, border_type, ctx);
}

kleidicv_error_t kleidicv_gpu_separable_filter_2d_u8_sme(const uint8_t *src, size_t src_stride, uint8_t *dst,
                                                         size_t dst_stride, size_t width, size_t height,
                                                         size_t channels, const uint8_t *kernel_x,
                                                         size_t kernel_width, const uint8_t *kernel_y,
                                                         size_t kernel_height, kleidicv_border_type_t border_type,
                                                         kleidicv_gpu_context_t *ctx) {
  return kleidicv_gpu_separable_filter_2d_u8(src, src_stride, dst, dst_stride, width, height, channels, kernel_x,
                                             kernel_width, kernel_y, kernel_height, border_type, ctx);
}

kleidicv_error_t kleidicv_gpu_separable_filter_2d_u16_sme(const uint16_t *src, size_t src_stride, uint16_t *dst,
                                                          size_t dst_stride, size_t width, size_t height,
                                                          size_t channels, const uint16_t *kernel_x,
                                                          size_t kernel_width, const uint16_t *kernel_y,
                                                          size_t kernel_height, kleidicv_border_type_t border_type,
                                                          kleidicv_gpu_context_t *ctx) {
  return kleidicv_gpu_separable_filter_2d_u16(src, src_stride, dst, dst_stride, width, height, channels, kernel_x,
                                              kernel_width, kernel_y, kernel_height, border_type, ctx);
}

kleidicv_error_t kleidicv_gpu_blur_and_downsample_u8_sme(const uint8_t *src, size_t src_stride, size_t src_width,
                                                         size_t src_height, uint8_t *dst, size_t dst_stride,
                                                         size_t channels, kleidicv_border_type_t border_type,
                                                         kleidicv_gpu_context_t *ctx) {
  return kleidicv_gpu_blur_and_downsample_u8(src, src_stride, src_width, src_height, dst, dst_stride, channels,
                                             border_type, ctx);
}

kleidicv_error_t kleidicv_gpu_sobel_3x3_horizontal_s16_u8_sme(const uint8_t *src, size_t src_stride, int16_t *dst,
                                                              size_t dst_stride, size_t width, size_t height,
                                                              size_t channels, kleidicv_gpu_context_t *ctx) {
  return kleidicv_gpu_sobel_3x3_horizontal_s16_u8(src, src_stride, dst, dst_stride, width, height, channels, ctx);
}

kleidicv_error_t kleidicv_gpu_sobel_3x3_vertical_s16_u8_sme(const uint8_t *src, size_t src_stride, int16_t *dst,
                                                            size_t dst_stride, size_t width, size_t height,
                                                            size_t channels, kleidicv_gpu_context_t *ctx) {
  return kleidicv_gpu_sobel_3x3_vertical_s16_u8(src, src_stride, dst, dst_stride, width, height, channels, ctx);
}

}  // extern "C"
