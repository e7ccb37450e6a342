// C-ABI of the median blur: kleidicv_median_blur_{s8,u8,u16,s16,u32,s32,f32}
// (kleidicv/src/filters/median_blur_api.cpp:42-242) with the checks of
// median_blur_is_implemented (kleidicv/include/kleidicv/filters/
// median_blur.h:148-193), in that order, then one launch on the context's
// stream.
#include <stdint.h>

#include "host.h"

namespace kcv {

constexpr uint64_t kMaxImagePixels = (1ull << 48) - 1;  // kleidicv.h:103

kleidicv_error_t validate_median(int elem, size_t es, const void *src, size_t src_stride,
                                 const void *dst, size_t dst_stride, size_t width, size_t height,
                                 size_t channels, size_t kernel_width, size_t kernel_height,
                                 int border, bool *work) {
  *work = false;
  // check_ptrs_strides_imagesizes (median_blur.h:148-158).
  if (!src) return KLEIDICV_ERROR_NULL_POINTER;
  if (height > 1 && src_stride % es != 0) return KLEIDICV_ERROR_ALIGNMENT;
  if (!dst) return KLEIDICV_ERROR_NULL_POINTER;
  if (height > 1 && dst_stride % es != 0) return KLEIDICV_ERROR_ALIGNMENT;
  size_t pixels;
  if (__builtin_mul_overflow(width, height, &pixels) || pixels > kMaxImagePixels)
    return KLEIDICV_ERROR_RANGE;
  // is_kernel_size_supported (:160-171) and the rest of :173-193.
  const size_t kmax = elem == MEDIAN_U8 ? 255 : 7;
  const bool kernel_ok = kernel_width == kernel_height && kernel_width >= 3 &&
                         kernel_width <= kmax && (kernel_width % 2) != 0;
  const bool border_ok = border == KLEIDICV_BORDER_TYPE_REPLICATE ||
                         border == KLEIDICV_BORDER_TYPE_REFLECT ||
                         border == KLEIDICV_BORDER_TYPE_WRAP ||
                         border == KLEIDICV_BORDER_TYPE_REVERSE;
  if (!(src != dst && channels <= KLEIDICV_GPU_MAXIMUM_CHANNEL_COUNT &&
        height >= kernel_height - 1 && width >= kernel_width - 1 && kernel_ok && border_ok))
    return KLEIDICV_ERROR_NOT_IMPLEMENTED;
  if (channels == 0 || width == 0 || height == 0) return KLEIDICV_OK;
  // 32-bit row and column indexing on the device (see the fused filters).
  if (width * channels * es > (size_t{1} << 30) || height > (size_t{1} << 30))
    return KLEIDICV_ERROR_RANGE;
  *work = true;
  return KLEIDICV_OK;
}

}  // namespace kcv

namespace {

using kcv::MedianElem;

kleidicv_error_t median_blur(MedianElem elem, size_t es, const void *src, size_t src_stride,
                             void *dst, size_t dst_stride, size_t width, size_t height,
                             size_t channels, size_t kernel_width, size_t kernel_height,
                             kleidicv_border_type_t border, kleidicv_gpu_context_t *ctx) {
  bool work = false;
  const kleidicv_error_t v =
      kcv::validate_median(elem, es, src, src_stride, dst, dst_stride, width, height, channels,
                           kernel_width, kernel_height, border, &work);
  if (v != KLEIDICV_OK || !work) return v;

  kleidicv_error_t e = kcv::resolve_context(ctx);
  if (e != KLEIDICV_OK) return e;
  kcv::DeviceGuard guard(ctx->device);
  kcv::MedianJob j;
  j.src = static_cast<const uint8_t *>(src);
  j.dst = static_cast<uint8_t *>(dst);
  j.src_stride = static_cast<int64_t>(src_stride);
  j.dst_stride = static_cast<int64_t>(dst_stride);
  j.width = static_cast<int32_t>(width);
  j.height = static_cast<int32_t>(height);
  j.channels = static_cast<int32_t>(channels);
  j.ksize = static_cast<int32_t>(kernel_width);
  j.border = static_cast<int32_t>(border);
  j.elem = elem;
  const cudaError_t ce = kcv::launch_median(j, ctx->stream);
  ctx->launches += 1;
  return kcv::cuda_status(ctx, ce);
}

}  // namespace

extern "C" {

#define KCV_MEDIAN_ENTRY(suffix, T, ELEM)                                                    \
  kleidicv_error_t kleidicv_gpu_median_blur_##suffix(                                        \
      const T *src, size_t src_stride, T *dst, size_t dst_stride, size_t width,              \
      size_t height, size_t channels, size_t kernel_width, size_t kernel_height,             \
      kleidicv_border_type_t border_type, kleidicv_gpu_context_t *ctx) {                     \
    return median_blur(kcv::ELEM, sizeof(T), src, src_stride, dst, dst_stride, width, height, \
                       channels, kernel_width, kernel_height, border_type, ctx);             \
  }

KCV_MEDIAN_ENTRY(s8, int8_t, MEDIAN_S8)
KCV_MEDIAN_ENTRY(u8, uint8_t, MEDIAN_U8)
KCV_MEDIAN_ENTRY(u16, uint16_t, MEDIAN_U16)
KCV_MEDIAN_ENTRY(s16, int16_t, MEDIAN_S16)
KCV_MEDIAN_ENTRY(u32, uint32_t, MEDIAN_U32)
KCV_MEDIAN_ENTRY(s32, int32_t, MEDIAN_S32)
KCV_MEDIAN_ENTRY(f32, float, MEDIAN_F32)

#undef KCV_MEDIAN_ENTRY

}  // extern "C"
