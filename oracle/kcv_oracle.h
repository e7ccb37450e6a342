/*
 * CPU oracle for the separable-filter hot path of KleidiCV.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links, loads or
 * calls this code; only tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline / --impl reference leg use it, as the checker or as the timed
 * CPU baseline ("port").
 *
 * It restates, in plain C, the integer arithmetic of (paths relative to the
 * KleidiCV project root):
 *   - kleidicv/src/filters/gaussian_blur_api.cpp:21-53 (validation + routing)
 *   - kleidicv/include/kleidicv/filters/gaussian_blur.h:38-95 (is_implemented,
 *     checks)
 *   - kleidicv/src/filters/gaussian_blur_fixed_neon.cpp:33-459 (binomial
 *     3/5/7/9 coefficient sets and shifts), :461-529 (sigma kernels,
 *     u8-rounded intermediate), :531-576 (copy fallback when mid weight is 256)
 *   - kleidicv/src/filters/gaussian_blur_arbitrary_neon.cpp:128-388 (odd
 *     kernel sizes 11..255, replicate border)
 *   - kleidicv/include/kleidicv/filters/sigma.h:16-79 (half-kernel generator)
 *   - kleidicv/src/filters/separable_filter_2d_neon.cpp:19-260 (u8/u16 5x5
 *     with saturation) and separable_filter_2d_api.cpp:12-31
 *   - kleidicv/src/filters/blur_and_downsample_neon.cpp:22-344 and
 *     kleidicv/include/kleidicv/workspace/blur_and_downsample_ws.h:42-111
 *   - kleidicv/include/kleidicv/workspace/border_{3x3,5x5,7x7,9x9,15x15,21x21}.h
 *     (border offset tables; restated as a single-fold index map, valid for
 *     sizes >= kernel_size - 1)
 *   - kleidicv/include/kleidicv/utils.h:379-430 (pointer/stride/size checks)
 *
 * Extension semantics that the reference does not define (CONSTANT border,
 * the s16 separable filter) are defined here and are "parity unpinned".
 */
#ifndef KCV_ORACLE_H
#define KCV_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  KO_OK = 0,
  KO_NOT_IMPLEMENTED = 1,
  KO_NULL_POINTER = 2,
  KO_RANGE = 3,
  KO_ALLOCATION = 4,
  KO_ALIGNMENT = 5,
};

enum {
  KO_BORDER_CONSTANT = 0,
  KO_BORDER_REPLICATE = 1,
  KO_BORDER_REFLECT = 2,
  KO_BORDER_WRAP = 3,
  KO_BORDER_REVERSE = 4,
  KO_BORDER_TRANSPARENT = 5,
  KO_BORDER_NONE = 6,
};

/* Half-kernel generator (sigma.h:27-79).  Returns 1 and fills half_size
 * weights, or returns 0 when all weight sits in the middle tap ("copy"). */
int ko_gaussian_half_kernel(uint8_t *half_kernel, size_t half_size,
                            float sigma);

/* Single-fold border map used by the fixed-size offset tables (and clamp for
 * the arbitrary path).  Returns -1 for CONSTANT outside [0, n). */
long ko_border_map(long i, long n, int border);

/* out[i * ksize + t] = ko_border_map(i + t - ksize / 2, n, border). */
void ko_border_table(int ksize, long n, int border, long *out);

/* Drop-in semantics.  `ext` = 0 reproduces the reference exactly (including
 * its error codes); `ext` = 1 additionally accepts KLEIDICV_BORDER_TYPE_CONSTANT
 * with `border_value` (extension, parity unpinned).  nthreads > 1 splits rows
 * into stripes over pthreads (same result; used for the CPU baseline). */
int ko_gaussian_blur_u8(const uint8_t *src, size_t src_stride, uint8_t *dst,
                        size_t dst_stride, size_t width, size_t height,
                        size_t channels, size_t kernel_width,
                        size_t kernel_height, float sigma_x, float sigma_y,
                        int border_type, int ext, int border_value,
                        int nthreads);

int ko_separable_filter_2d_u8(const uint8_t *src, size_t src_stride,
                              uint8_t *dst, size_t dst_stride, size_t width,
                              size_t height, size_t channels,
                              const uint8_t *kernel_x, size_t kernel_width,
                              const uint8_t *kernel_y, size_t kernel_height,
                              int border_type, int ext, int border_value,
                              int nthreads);

int ko_separable_filter_2d_u16(const uint16_t *src, size_t src_stride,
                               uint16_t *dst, size_t dst_stride, size_t width,
                               size_t height, size_t channels,
                               const uint16_t *kernel_x, size_t kernel_width,
                               const uint16_t *kernel_y, size_t kernel_height,
                               int border_type, int ext, int border_value,
                               int nthreads);

/* s16 has no reference definition: always extension semantics. */
int ko_separable_filter_2d_s16(const int16_t *src, size_t src_stride,
                               int16_t *dst, size_t dst_stride, size_t width,
                               size_t height, size_t channels,
                               const int16_t *kernel_x, size_t kernel_width,
                               const int16_t *kernel_y, size_t kernel_height,
                               int border_type, int border_value,
                               int nthreads);

int ko_blur_and_downsample_u8(const uint8_t *src, size_t src_stride,
                              size_t src_width, size_t src_height,
                              uint8_t *dst, size_t dst_stride, size_t channels,
                              int border_type, int ext, int border_value,
                              int nthreads);

/* 3x3 Sobel derivatives, u8 -> s16, REPLICATE border (sobel_api.cpp:22-76):
 * horizontal = [1 2 1]^T x [-1 0 1], vertical = [-1 0 1]^T x [1 2 1]. */
int ko_sobel_3x3_horizontal_s16_u8(const uint8_t *src, size_t src_stride,
                                   int16_t *dst, size_t dst_stride,
                                   size_t width, size_t height,
                                   size_t channels, int nthreads);
int ko_sobel_3x3_vertical_s16_u8(const uint8_t *src, size_t src_stride,
                                 int16_t *dst, size_t dst_stride, size_t width,
                                 size_t height, size_t channels, int nthreads);

#ifdef __cplusplus
}
#endif

#endif /* KCV_ORACLE_H */
