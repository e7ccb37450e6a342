// OpenCV custom-HAL shim (include/kleidicv_gpu_hal.h): the acceptance rules,
// border mapping and error mapping of KleidiCV's OpenCV adapter
// (adapters/opencv/kleidicv_hal.cpp), routed to the GPU entry points.  Host
// images are staged through device memory on the calling thread's default
// context; every call returns only when the result is in `dst`.
#include "../../include/kleidicv_gpu_hal.h"

#include <cuda_runtime.h>

#include <functional>

#include "host.h"

namespace {

// The OpenCV HAL ABI values used here (opencv2/core/hal/interface.h).
constexpr int kHalOk = 0;
constexpr int kHalNotImplemented = 1;
constexpr int kHalUnknown = -1;
constexpr int kCv8U = 0, kCv16U = 2, kCv16S = 3;
constexpr int kHalBorderConstant = 0, kHalBorderReplicate = 1, kHalBorderReflect = 2,
              kHalBorderWrap = 3, kHalBorderReflect101 = 4, kHalBorderTransparent = 5,
              kHalBorderIsolated = 16;
int mat_depth(int type) { return type & 7; }
int mat_channels(int type) { return ((type >> 3) & 511) + 1; }

// convert_error (kleidicv_hal.cpp:78-91); every GPU-side failure (no device,
// CUDA error, timeout) is an error OpenCV reports, never a silent fallback.
int convert_error(kleidicv_error_t e) {
  switch (e) {
    case KLEIDICV_OK: return kHalOk;
    case KLEIDICV_ERROR_NOT_IMPLEMENTED: return kHalNotImplemented;
    case KLEIDICV_ERROR_ALIGNMENT: return kHalNotImplemented;
    default: return kHalUnknown;
  }
}

// from_opencv for border types (kleidicv_hal.cpp:405-435): exact values only
// (a border OR-ed with BORDER_ISOLATED is not mapped).
bool from_opencv(int cv_border, kleidicv_border_type_t &b) {
  switch (cv_border) {
    case kHalBorderConstant: b = KLEIDICV_BORDER_TYPE_CONSTANT; return true;
    case kHalBorderReplicate: b = KLEIDICV_BORDER_TYPE_REPLICATE; return true;
    case kHalBorderReflect: b = KLEIDICV_BORDER_TYPE_REFLECT; return true;
    case kHalBorderReflect101: b = KLEIDICV_BORDER_TYPE_REVERSE; return true;
    case kHalBorderWrap: b = KLEIDICV_BORDER_TYPE_WRAP; return true;
    case kHalBorderTransparent: b = KLEIDICV_BORDER_TYPE_TRANSPARENT; return true;
    case kHalBorderIsolated: b = KLEIDICV_BORDER_TYPE_NONE; return true;
    default: return false;
  }
}

bool is_device_pointer(const void *p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();  // clear the sticky-free error of an unknown pointer
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

struct Image {
  const void *ptr;
  size_t step, row_bytes, rows;
};

// Runs `op(src, src_step, dst, dst_step)` on device pointers, staging a host
// source / destination through device buffers (rows packed at a 256-byte
// pitch), then waits for the result.  `validation` is the entry's own check
// with the caller's pointers (`p` its outcome): nothing is copied for a call
// it rejects or that has nothing to compute.
int run_staged(kleidicv_error_t validation, const kcv::Prepared &p, Image src, Image dst,
               const std::function<kleidicv_error_t(const void *, size_t, void *, size_t,
                                                    kleidicv_gpu_context_t *)> &op) {
  if (validation != KLEIDICV_OK) return convert_error(validation);
  if (p.kind == kcv::Prepared::NOTHING) return kHalOk;
  // A single-row image may come with any stride (the reference ignores it).
  if (src.rows <= 1) src.step = src.row_bytes;
  if (dst.rows <= 1) dst.step = dst.row_bytes;
  kleidicv_gpu_context_t *ctx = nullptr;
  kleidicv_error_t e = kcv::resolve_context(ctx);
  if (e != KLEIDICV_OK) return convert_error(e);
  kcv::DeviceGuard guard(ctx->device);
  const bool src_dev = is_device_pointer(src.ptr), dst_dev = is_device_pointer(dst.ptr);
  auto pitch_of = [](size_t row_bytes) { return (row_bytes + 255) / 256 * 256; };
  const size_t sp = src_dev ? src.step : pitch_of(src.row_bytes);
  const size_t dp = dst_dev ? dst.step : pitch_of(dst.row_bytes);
  const size_t sbytes = src_dev ? 0 : sp * src.rows, dbytes = dst_dev ? 0 : dp * dst.rows;
  void *sbuf = sbytes ? kcv::ctx_alloc(ctx, sbytes) : nullptr;
  void *dbuf = dbytes ? kcv::ctx_alloc(ctx, dbytes) : nullptr;
  if ((sbytes && !sbuf) || (dbytes && !dbuf)) {
    kcv::ctx_free(ctx, sbuf, sbytes);
    kcv::ctx_free(ctx, dbuf, dbytes);
    return convert_error(KLEIDICV_ERROR_ALLOCATION);
  }
  cudaError_t ce = cudaSuccess;
  if (!src_dev)
    ce = cudaMemcpy2DAsync(sbuf, sp, src.ptr, src.step, src.row_bytes, src.rows,
                           cudaMemcpyHostToDevice, ctx->stream);
  if (ce == cudaSuccess) {
    e = op(src_dev ? src.ptr : sbuf, sp, dst_dev ? const_cast<void *>(dst.ptr) : dbuf, dp, ctx);
    if (e == KLEIDICV_OK && !dst_dev)
      ce = cudaMemcpy2DAsync(const_cast<void *>(dst.ptr), dst.step, dbuf, dp, dst.row_bytes,
                             dst.rows, cudaMemcpyDeviceToHost, ctx->stream);
  }
  kcv::ctx_free(ctx, sbuf, sbytes);
  kcv::ctx_free(ctx, dbuf, dbytes);
  const kleidicv_error_t se = kleidicv_gpu_context_synchronize(ctx);
  if (ce != cudaSuccess) return convert_error(kcv::cuda_status(ctx, ce));
  if (e != KLEIDICV_OK) return convert_error(e);
  return convert_error(se);
}

}  // namespace

extern "C" {

int kleidicv_gpu_hal_separable_filter_2d(
    const unsigned char *src_data, size_t src_step, int src_type, unsigned char *dst_data,
    size_t dst_step, int dst_type, int width, int height, int full_width, int full_height,
    int offset_x, int offset_y, const unsigned char *kernelx_data, int kernelx_len,
    const unsigned char *kernely_data, int kernely_len, int kernel_type, int anchor_x,
    int anchor_y, double delta, int border_type) {
  // kleidicv_hal.cpp:459-515, in the same order.
  const int margin_right = full_width - width - offset_x;
  const int margin_bottom = full_height - height - offset_y;
  if (offset_x != 0 || offset_y != 0 || margin_right != 0 || margin_bottom != 0)
    return kHalNotImplemented;
  if (src_data == dst_data) return kHalNotImplemented;
  if (src_type != dst_type) return kHalNotImplemented;
  if (mat_depth(src_type) != mat_depth(kernel_type)) return kHalNotImplemented;
  if (mat_channels(kernel_type) != 1) return kHalNotImplemented;
  const int depth = mat_depth(src_type);
  if (depth != kCv8U && depth != kCv16U) return kHalNotImplemented;
  kleidicv_border_type_t b;
  if (!from_opencv(border_type, b)) return kHalNotImplemented;
  if (b != KLEIDICV_BORDER_TYPE_REPLICATE && b != KLEIDICV_BORDER_TYPE_REFLECT &&
      b != KLEIDICV_BORDER_TYPE_WRAP && b != KLEIDICV_BORDER_TYPE_REVERSE)
    return kHalNotImplemented;
  if (anchor_x > -1 && anchor_x != (kernelx_len >> 1)) return kHalNotImplemented;
  if (anchor_y > -1 && anchor_y != (kernely_len >> 1)) return kHalNotImplemented;
  if (delta != 0.0) return kHalNotImplemented;

  const size_t cn = static_cast<size_t>(mat_channels(src_type));
  const size_t w = static_cast<size_t>(width), h = static_cast<size_t>(height);
  const size_t kw = static_cast<size_t>(kernelx_len), kh = static_cast<size_t>(kernely_len);
  const int elem = depth == kCv8U ? 1 : 2;
  kcv::Prepared p;
  const kleidicv_error_t v = kcv::prepare_separable(elem, src_data, src_step, dst_data, dst_step,
                                                    w, h, cn, kernelx_data, kw, kernely_data, kh,
                                                    b, false, 0, &p);
  const size_t rb = w * cn * static_cast<size_t>(elem);
  return run_staged(v, p, {src_data, src_step, rb, h}, {dst_data, dst_step, rb, h},
                    [&](const void *s, size_t ss, void *d, size_t ds, kleidicv_gpu_context_t *c) {
                      if (elem == 1)
                        return kleidicv_gpu_separable_filter_2d_u8(
                            static_cast<const uint8_t *>(s), ss, static_cast<uint8_t *>(d), ds, w,
                            h, cn, kernelx_data, kw, kernely_data, kh, b, c);
                      return kleidicv_gpu_separable_filter_2d_u16(
                          static_cast<const uint16_t *>(s), ss, static_cast<uint16_t *>(d), ds, w,
                          h, cn, reinterpret_cast<const uint16_t *>(kernelx_data), kw,
                          reinterpret_cast<const uint16_t *>(kernely_data), kh, b, c);
                    });
}

int kleidicv_gpu_hal_gaussian_blur(
    const unsigned char *src_data, size_t src_step, unsigned char *dst_data, size_t dst_step,
    int width, int height, int depth, int cn, size_t margin_left, size_t margin_top,
    size_t margin_right, size_t margin_bottom, size_t kernel_width, size_t kernel_height,
    double sigma_x, double sigma_y, int border_type) {
  // kleidicv_hal.cpp:591-620.
  if (src_data == dst_data) return kHalNotImplemented;
  if (margin_left != 0 || margin_top != 0 || margin_right != 0 || margin_bottom != 0)
    return kHalNotImplemented;
  if (depth != kCv8U) return kHalNotImplemented;
  kleidicv_border_type_t b;
  if (!from_opencv(border_type, b)) return kHalNotImplemented;
  const size_t w = static_cast<size_t>(width), h = static_cast<size_t>(height);
  const size_t c = static_cast<size_t>(cn);
  const float sx = static_cast<float>(sigma_x), sy = static_cast<float>(sigma_y);
  kcv::Prepared p;
  const kleidicv_error_t v = kcv::prepare_gaussian(src_data, src_step, dst_data, dst_step, w, h, c,
                                                   kernel_width, kernel_height, sx, sy, b, false,
                                                   0, &p);
  return run_staged(v, p, {src_data, src_step, w * c, h}, {dst_data, dst_step, w * c, h},
                    [&](const void *s, size_t ss, void *d, size_t ds, kleidicv_gpu_context_t *x) {
                      return kleidicv_gpu_gaussian_blur_u8(static_cast<const uint8_t *>(s), ss,
                                                           static_cast<uint8_t *>(d), ds, w, h, c,
                                                           kernel_width, kernel_height, sx, sy, b,
                                                           x);
                    });
}

int kleidicv_gpu_hal_gaussian_blur_binomial(
    const unsigned char *src_data, size_t src_step, unsigned char *dst_data, size_t dst_step,
    int width, int height, int depth, int cn, size_t margin_left, size_t margin_top,
    size_t margin_right, size_t margin_bottom, size_t kernel_size, int border_type) {
  // kleidicv_hal.cpp:556-583: the generic call with sigma 0.
  return kleidicv_gpu_hal_gaussian_blur(src_data, src_step, dst_data, dst_step, width, height,
                                        depth, cn, margin_left, margin_top, margin_right,
                                        margin_bottom, kernel_size, kernel_size, 0.0, 0.0,
                                        border_type);
}

int kleidicv_gpu_hal_pyrdown(const unsigned char *src_data, size_t src_step, int src_width,
                             int src_height, unsigned char *dst_data, size_t dst_step,
                             int dst_width, int dst_height, int depth, int cn, int border_type) {
  // kleidicv_hal.cpp:1565-1591.
  if (src_data == dst_data) return kHalNotImplemented;
  if (depth != kCv8U) return kHalNotImplemented;
  if (dst_width != (src_width + 1) / 2 || dst_height != (src_height + 1) / 2)
    return kHalNotImplemented;
  kleidicv_border_type_t b;
  if (!from_opencv(border_type, b)) return kHalNotImplemented;
  const size_t sw = static_cast<size_t>(src_width), sh = static_cast<size_t>(src_height);
  const size_t c = static_cast<size_t>(cn);
  kcv::Prepared p;
  const kleidicv_error_t v =
      kcv::prepare_blurdown(src_data, src_step, sw, sh, dst_data, dst_step, c, b, false, 0, &p);
  const size_t dw = (sw + 1) / 2, dh = (sh + 1) / 2;
  return run_staged(v, p, {src_data, src_step, sw * c, sh}, {dst_data, dst_step, dw * c, dh},
                    [&](const void *s, size_t ss, void *d, size_t ds, kleidicv_gpu_context_t *x) {
                      return kleidicv_gpu_blur_and_downsample_u8(static_cast<const uint8_t *>(s),
                                                                 ss, sw, sh,
                                                                 static_cast<uint8_t *>(d), ds, c,
                                                                 b, x);
                    });
}

int kleidicv_gpu_hal_sobel(const unsigned char *src_data, size_t src_step,
                           unsigned char *dst_data, size_t dst_step, int width, int height,
                           int src_depth, int dst_depth, int cn, int margin_left,
                           int margin_top, int margin_right, int margin_bottom, int dx, int dy,
                           int ksize, double scale, double delta, int border_type) {
  // kleidicv_hal.cpp:825-878, in the same order.
  if (src_data == dst_data) return kHalNotImplemented;
  if (src_depth != kCv8U) return kHalNotImplemented;
  if (dst_depth != kCv16S) return kHalNotImplemented;
  if (ksize != 3) return kHalNotImplemented;
  if (width < 3 || height < 3) return kHalNotImplemented;
  if (scale != 1.0) return kHalNotImplemented;
  if (delta != 0.0) return kHalNotImplemented;
  if (border_type != kHalBorderReplicate) return kHalNotImplemented;
  if (margin_left || margin_top || margin_right || margin_bottom) return kHalNotImplemented;
  const bool horizontal = dx == 1 && dy == 0;
  if (!horizontal && !(dx == 0 && dy == 1)) return kHalNotImplemented;
  const size_t w = static_cast<size_t>(width), h = static_cast<size_t>(height);
  const size_t c = static_cast<size_t>(cn);
  int16_t *dst16 = reinterpret_cast<int16_t *>(dst_data);
  kcv::Prepared p;
  const kleidicv_error_t v =
      kcv::prepare_sobel(horizontal, src_data, src_step, dst16, dst_step, w, h, c, &p);
  return run_staged(v, p, {src_data, src_step, w * c, h}, {dst_data, dst_step, 2 * w * c, h},
                    [&](const void *s, size_t ss, void *d, size_t ds, kleidicv_gpu_context_t *x) {
                      const uint8_t *su = static_cast<const uint8_t *>(s);
                      int16_t *di = static_cast<int16_t *>(d);
                      return horizontal
                                 ? kleidicv_gpu_sobel_3x3_horizontal_s16_u8(su, ss, di, ds, w, h, c, x)
                                 : kleidicv_gpu_sobel_3x3_vertical_s16_u8(su, ss, di, ds, w, h, c, x);
                    });
}

}  // extern "C"
