// Lucas-Kanade pyramid builder on the GPU: the image and Scharr pyramids of
// kleidicv_build_optical_flow_pyr_lk_pyramid
// (kleidicv/include/kleidicv/analysis/build_optical_flow_pyr_lk_pyramid.h:306-383).
//
// Every level is an image with a reflect-101 border of (window_width,
// window_height) pixels and the interleaved (dx, dy) Scharr derivatives of
// that image (s16, 2 x channels per pixel) with a zero halo of the same size.
// Level l >= 1 is blur_and_downsample (REVERSE) of level l - 1 through the
// blur-and-downsample call path (the pyramid kernel), written straight into
// the level's interior; one "finish" kernel per
// level then writes the border (and, for level 0, the interior copy) and the
// Scharr derivatives, reading the interior with the reflect-101 index map
// instead of waiting for the border to exist.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "../../include/kleidicv_gpu.h"
#include "host.h"
#include "launch.h"

namespace kcv {
namespace {

constexpr size_t kMaxLkWindow = 2047;  // KLEIDICV_MAX_OPTICAL_FLOW_PYR_LK_WINDOW_SIZE

__device__ __forceinline__ int reflect_101(int i, int n) {
  if (n <= 1) return 0;
  while (i < 0 || i >= n) i = i < 0 ? -i : 2 * n - i - 2;
  return i;
}

// One thread per pixel of the bordered level: copies the mapped image pixel
// (the interior only when `copy_interior`) and, inside the image, computes the
// Scharr pair of every channel from the reflect-101 3x3 neighbourhood.
__global__ void __launch_bounds__(256) lk_finish_level(const uint8_t *src, int64_t src_stride,
                                                       uint8_t *img, int64_t img_stride,
                                                       int16_t *sch, int64_t sch_stride, int w,
                                                       int h, int c, int bw, int bh,
                                                       int copy_interior) {
  const int bx = blockIdx.x * blockDim.x + threadIdx.x;  // column of the bordered image
  if (bx >= w + 2 * bw) return;
  for (int by = blockIdx.y; by < h + 2 * bh; by += gridDim.y) {  // rows of the bordered image
  const int x = bx - bw, y = by - bh;
  const bool inside = x >= 0 && x < w && y >= 0 && y < h;
  const int sx = reflect_101(x, w), sy = reflect_101(y, h);
  uint8_t *dpix = img + static_cast<int64_t>(y) * img_stride + static_cast<int64_t>(x) * c;
  const uint8_t *spix = src + static_cast<int64_t>(sy) * src_stride + static_cast<int64_t>(sx) * c;
  if (!inside || copy_interior)
    for (int ch = 0; ch < c; ++ch) dpix[ch] = spix[ch];
  if (!inside) continue;
  const int xl = reflect_101(x - 1, w), xr = reflect_101(x + 1, w);
  const int yu = reflect_101(y - 1, h), yd = reflect_101(y + 1, h);
  const uint8_t *ru = src + static_cast<int64_t>(yu) * src_stride;
  const uint8_t *rm = src + static_cast<int64_t>(y) * src_stride;
  const uint8_t *rd = src + static_cast<int64_t>(yd) * src_stride;
  int16_t *out = reinterpret_cast<int16_t *>(reinterpret_cast<uint8_t *>(sch) +
                                             static_cast<int64_t>(y) * sch_stride) +
                 static_cast<int64_t>(x) * c * 2;
  for (int ch = 0; ch < c; ++ch) {
    const int ul = ru[xl * c + ch], um = ru[x * c + ch], ur = ru[xr * c + ch];
    const int ml = rm[xl * c + ch], mr = rm[xr * c + ch];
    const int dl = rd[xl * c + ch], dm = rd[x * c + ch], dr = rd[xr * c + ch];
    // Scharr: |dx|, |dy| <= 16 * 255, inside int16.
    const int dx = 3 * (ur - ul) + 10 * (mr - ml) + 3 * (dr - dl);
    const int dy = 3 * (dl - ul) + 10 * (dm - um) + 3 * (dr - ur);
    out[2 * ch] = static_cast<int16_t>(dx);
    out[2 * ch + 1] = static_cast<int16_t>(dy);
  }
  }
}

size_t round_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

}  // namespace
}  // namespace kcv

using namespace kcv;

struct kleidicv_gpu_lk_pyramid {
  kleidicv_gpu_context *ctx = nullptr;
  uint8_t *dmem = nullptr;
  size_t dmem_bytes = 0;
  size_t channels = 0, border_w = 0, border_h = 0;
  struct Level {
    size_t width, height, image_stride, scharr_stride;
    uint8_t *image;   // interior (device)
    int16_t *scharr;  // interior (device)
  };
  std::vector<Level> levels;
};

extern "C" {

kleidicv_error_t kleidicv_gpu_build_optical_flow_pyr_lk_pyramid(
    kleidicv_gpu_lk_pyramid_t **pyramid, const uint8_t *src, size_t src_stride, size_t width,
    size_t height, size_t channels, size_t level_count, size_t window_width, size_t window_height,
    kleidicv_gpu_context_t *ctx) {
  // build_optical_flow_pyr_lk_pyramid_api.cpp:13-26, then
  // validate_and_compute_build_optical_flow_pyr_lk_levels (:18-58).
  if (!pyramid) return KLEIDICV_ERROR_NULL_POINTER;
  if (!src) return KLEIDICV_ERROR_NULL_POINTER;
  size_t pixels;
  if (__builtin_mul_overflow(width, height, &pixels) || pixels > ((1ull << 48) - 1))
    return KLEIDICV_ERROR_RANGE;
  if (width == 0 || height == 0 || channels == 0 || channels > 4 || level_count == 0 ||
      window_width <= 2 || window_height <= 2 || window_width > kMaxLkWindow ||
      window_height > kMaxLkWindow)
    return KLEIDICV_ERROR_RANGE;
  if (height > 1 && src_stride < width * channels) return KLEIDICV_ERROR_RANGE;
  size_t n = 0, lw = width, lh = height;
  std::vector<std::pair<size_t, size_t>> sizes;
  for (size_t r = 0; r < level_count; ++r) {
    ++n;
    sizes.emplace_back(lw, lh);
    const size_t nw = (lw + 1) / 2, nh = (lh + 1) / 2;
    if (nw <= window_width || nh <= window_height) break;
    lw = nw;
    lh = nh;
  }
  // 32-bit row and column indexing on the device (bordered level 0, Scharr rows).
  if ((width + 2 * window_width) * channels * 4 > (size_t{1} << 30) ||
      height + 2 * window_height > (size_t{1} << 30))
    return KLEIDICV_ERROR_RANGE;
  kleidicv_error_t e = resolve_context(ctx);
  if (e != KLEIDICV_OK) return e;
  DeviceGuard guard(ctx->device);

  auto *p = new kleidicv_gpu_lk_pyramid();
  p->ctx = ctx;
  p->channels = channels;
  p->border_w = window_width;
  p->border_h = window_height;
  // Layout per level: [image rows][scharr rows], each 256-byte aligned; the
  // image interior starts 16-byte aligned (left border rounded up) so that
  // the next level's blur-and-downsample reads it through TMA.
  const size_t lead = round_up(window_width * channels, 16);
  std::vector<size_t> img_off(n), sch_off(n);
  size_t total = 0;
  for (size_t l = 0; l < n; ++l) {
    const size_t w = sizes[l].first, h = sizes[l].second;
    const size_t istride = round_up(lead + (w + window_width) * channels, 16);
    const size_t sstride = round_up((w + 2 * window_width) * channels * 2 * sizeof(int16_t), 16);
    img_off[l] = total;
    total = round_up(total + istride * (h + 2 * window_height), 256);
    sch_off[l] = total;
    total = round_up(total + sstride * (h + 2 * window_height), 256);
    kleidicv_gpu_lk_pyramid::Level lv{w, h, istride, sstride, nullptr, nullptr};
    p->levels.push_back(lv);
  }
  p->dmem = static_cast<uint8_t *>(ctx_alloc(ctx, total));
  if (!p->dmem) {
    delete p;
    return KLEIDICV_ERROR_ALLOCATION;
  }
  p->dmem_bytes = total;
  cudaError_t ce = cudaMemsetAsync(p->dmem, 0, total, ctx->stream);  // Scharr halos are zero
  for (size_t l = 0; l < n && ce == cudaSuccess; ++l) {
    auto &lv = p->levels[l];
    lv.image = p->dmem + img_off[l] + window_height * lv.image_stride + lead;
    lv.scharr = reinterpret_cast<int16_t *>(p->dmem + sch_off[l] + window_height * lv.scharr_stride +
                                            window_width * channels * 2 * sizeof(int16_t));
    const uint8_t *lsrc = src;
    size_t lsrc_stride = src_stride;
    if (l > 0) {
      const auto &prev = p->levels[l - 1];
      Prepared pr;
      e = prepare_blurdown(prev.image, prev.image_stride, prev.width, prev.height, lv.image,
                           lv.image_stride, channels, BORDER_REVERSE, false, 0, &pr);
      if (e == KLEIDICV_OK) e = execute(ctx, pr);
      if (e != KLEIDICV_OK) break;
      lsrc = lv.image;
      lsrc_stride = lv.image_stride;
    }
    const int bw = static_cast<int>(window_width), bh = static_cast<int>(window_height);
    dim3 grid(static_cast<unsigned>((lv.width + 2 * window_width + 255) / 256),
              static_cast<unsigned>(std::min<size_t>(lv.height + 2 * window_height, 65535)));
    lk_finish_level<<<grid, 256, 0, ctx->stream>>>(
        lsrc, static_cast<int64_t>(lsrc_stride), lv.image, static_cast<int64_t>(lv.image_stride),
        lv.scharr, static_cast<int64_t>(lv.scharr_stride), static_cast<int>(lv.width),
        static_cast<int>(lv.height), static_cast<int>(channels), bw, bh, l == 0 ? 1 : 0);
    ce = cudaGetLastError();
    ctx->launches += 1;
  }
  if (e == KLEIDICV_OK && ce != cudaSuccess) e = cuda_status(ctx, ce);
  if (e != KLEIDICV_OK) {
    ctx_free(ctx, p->dmem, p->dmem_bytes);
    delete p;
    return e;
  }
  *pyramid = p;
  return KLEIDICV_OK;
}

kleidicv_error_t kleidicv_gpu_optical_flow_pyr_lk_pyramid_release(kleidicv_gpu_lk_pyramid_t *p) {
  if (!p) return KLEIDICV_ERROR_NULL_POINTER;
  DeviceGuard guard(p->ctx->device);
  ctx_free(p->ctx, p->dmem, p->dmem_bytes);  // stream-ordered after the builds
  delete p;
  return KLEIDICV_OK;
}

size_t kleidicv_gpu_lk_pyramid_level_count(const kleidicv_gpu_lk_pyramid_t *p) {
  return p ? p->levels.size() : 0;
}

kleidicv_error_t kleidicv_gpu_lk_pyramid_level(const kleidicv_gpu_lk_pyramid_t *p, size_t level,
                                               size_t *width, size_t *height,
                                               const uint8_t **image, size_t *image_stride,
                                               const int16_t **scharr, size_t *scharr_stride,
                                               size_t *border_width, size_t *border_height) {
  if (!p) return KLEIDICV_ERROR_NULL_POINTER;
  if (level >= p->levels.size()) return KLEIDICV_ERROR_RANGE;
  const auto &lv = p->levels[level];
  if (width) *width = lv.width;
  if (height) *height = lv.height;
  if (image) *image = lv.image;
  if (image_stride) *image_stride = lv.image_stride;
  if (scharr) *scharr = lv.scharr;
  if (scharr_stride) *scharr_stride = lv.scharr_stride;
  if (border_width) *border_width = p->border_w;
  if (border_height) *border_height = p->border_h;
  return KLEIDICV_OK;
}

}  // extern "C"
