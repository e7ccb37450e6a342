// C-ABI of the GB300 separable-filter library: validation in the reference's
// order, request preparation (weights, routing, tiling, TMA descriptors) and
// dispatch onto the context's stream.
#include <cudaTypedefs.h>
#include <string.h>

#include <algorithm>
#include <numeric>
#include <mutex>

#include "host.h"
#include "tune_table.h"

namespace kcv {

namespace {

constexpr uint64_t kMaxImagePixels = (1ull << 48) - 1;  // kleidicv.h:103
constexpr size_t kMaxChannels = 4;                      // kleidicv.h:110

bool fixed_border(int b) {
  return b == BORDER_REPLICATE || b == BORDER_REFLECT || b == BORDER_WRAP || b == BORDER_REVERSE;
}
// get_fixed_border_type (workspace/border_types.h:21-35); the _ex entry
// points additionally accept CONSTANT.
bool border_supported(int b, bool ext) { return fixed_border(b) || (ext && b == BORDER_CONSTANT); }

// CHECK_IMAGE_SIZE (utils.h:419-430).
bool image_size_ok(size_t w, size_t h) {
  size_t n;
  if (__builtin_mul_overflow(w, h, &n)) return false;
  return n <= kMaxImagePixels;
}

// The kernels index rows and columns in 32-bit arithmetic: a row of more than
// 2^30 bytes or more than 2^30 rows (images the reference accepts up to 2^48
// pixels, but no GPU holds as one row) is refused with RANGE instead of being
// processed wrongly.
bool device_dims_ok(size_t row_bytes, size_t height) {
  return row_bytes <= (size_t{1} << 30) && height <= (size_t{1} << 30);
}

// check_pointer_and_stride for 2-byte types (utils.h:379-390).
bool stride_misaligned(size_t stride, size_t height, size_t elem) {
  return height > 1 && (stride % elem) != 0;
}

// gaussian_blur_is_implemented (filters/gaussian_blur.h:38-82).
bool gaussian_is_implemented(size_t w, size_t h, size_t kw, size_t kh, float sx, float sy,
                             size_t c, int border, bool ext) {
  if (kw != kh) return false;
  if (kw < 3 || kw > 255) return false;
  if ((kw & 1) != 1) return false;
  if (!(sx == sy)) return false;
  if (w < kw - 1 || h < kw - 1) return false;
  if (c > kMaxChannels) return false;
  if (kw > 9 && kw != 15 && kw != 21) {
    if (border != BORDER_REPLICATE && !ext) return false;
    const size_t margin = kw / 2;
    const size_t aligned = (margin + 7) / 8 * 8;
    if (w < aligned + margin) return false;
  }
  return true;
}

int binomial_coef(int k, int i) {
  static const int c3[] = {1, 2, 1}, c5[] = {1, 4, 6, 4, 1}, c7[] = {2, 7, 14, 18, 14, 7, 2},
                   c9[] = {4, 13, 30, 51, 60, 51, 30, 13, 4};
  switch (k) {
    case 3: return c3[i];
    case 5: return c5[i];
    case 7: return c7[i];
    default: return c9[i];
  }
}

void fill_common(FilterJob &j, const void *src, size_t src_stride, void *dst, size_t dst_stride,
                 size_t w, size_t h, size_t c, int border, int border_value) {
  memset(&j, 0, sizeof(j));
  j.src = static_cast<const uint8_t *>(src);
  j.dst = static_cast<uint8_t *>(dst);
  j.src_stride = static_cast<int64_t>(src_stride);
  j.dst_stride = static_cast<int64_t>(dst_stride);
  j.width = static_cast<int32_t>(w);
  j.height = static_cast<int32_t>(h);
  j.channels = static_cast<int32_t>(c);
  j.out_width = static_cast<int32_t>(w);
  j.out_height = static_cast<int32_t>(h);
  j.border = border;
  j.border_value = border_value;
}

int elem_size(int mode) { return (mode == MODE_SEP_U16 || mode == MODE_SEP_S16) ? 2 : 1; }

int halo_chunks(const FilterJob &j) {
  const int halo_elems = j.mode == MODE_BLURDOWN ? 2 * j.channels + 2 : (j.ksize / 2) * j.channels;
  return (halo_elems * elem_size(j.mode) + kChunk - 1) / kChunk;
}

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return static_cast<PFN_cuTensorMapEncodeTiled_v12000>(nullptr);
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }();
  return fn;
}

}  // namespace

// ---------------------------------------------------------------------------
kleidicv_error_t prepare_gaussian(const uint8_t *src, size_t src_stride, uint8_t *dst,
                                  size_t dst_stride, size_t width, size_t height,
                                  size_t channels, size_t kernel_width, size_t kernel_height,
                                  float sigma_x, float sigma_y, int border, bool ext,
                                  int border_value, Prepared *out) {
  // gaussian_blur_api.cpp:28-37, then gaussian_blur_checks (gaussian_blur.h:86-95)
  if (!border_supported(border, ext)) return KLEIDICV_ERROR_NOT_IMPLEMENTED;
  if (!gaussian_is_implemented(width, height, kernel_width, kernel_height, sigma_x, sigma_y,
                               channels, border, ext))
    return KLEIDICV_ERROR_NOT_IMPLEMENTED;
  if (!src || !dst) return KLEIDICV_ERROR_NULL_POINTER;
  if (!image_size_ok(width, height)) return KLEIDICV_ERROR_RANGE;
  if (!device_dims_ok(width * channels, height)) return KLEIDICV_ERROR_RANGE;

  *out = Prepared{};
  if (channels == 0) return KLEIDICV_OK;
  const int k = static_cast<int>(kernel_width);
  const bool fixed = k <= 9 || k == 15 || k == 21;
  if (fixed && k <= 9 && sigma_x == 0.0f) {  // gaussian_blur_fixed_neon.cpp:633-637
    out->kind = Prepared::FUSED;
    FilterJob &j = out->fused;
    fill_common(j, src, src_stride, dst, dst_stride, width, height, channels, border,
                border_value & 0xFF);
    j.mode = MODE_BINOM;
    j.ksize = k;
    for (int t = 0; t < k; ++t) j.wy[t] = j.wx[t] = binomial_coef(k, t);
    return KLEIDICV_OK;
  }
  uint8_t half[128];
  if (!gaussian_half_kernel(kernel_width, sigma_x, half)) {
    out->kind = Prepared::COPY;
    out->src = src;
    out->src_stride = src_stride;
    out->dst = dst;
    out->dst_stride = dst_stride;
    out->row_bytes = width * channels;
    out->rows = height;
    return KLEIDICV_OK;
  }
  const int r = k / 2;
  int sum = half[r];
  for (int i = 0; i < r; ++i) sum += 2 * half[i];
  if (fixed && sum == 256) {
    out->kind = Prepared::FUSED;
    FilterJob &j = out->fused;
    fill_common(j, src, src_stride, dst, dst_stride, width, height, channels, border,
                border_value & 0xFF);
    j.mode = MODE_SIGMA;
    j.ksize = k;
    for (int t = 0; t < k; ++t) j.wy[t] = j.wx[t] = half[t <= r ? t : k - 1 - t];
    return KLEIDICV_OK;
  }
  out->kind = Prepared::GENERIC;
  GenericJob &g = out->generic;
  memset(&g, 0, sizeof(g));
  g.src = src;
  g.dst = dst;
  g.src_stride = static_cast<int64_t>(src_stride);
  g.dst_stride = static_cast<int64_t>(dst_stride);
  g.width = static_cast<int32_t>(width);
  g.height = static_cast<int32_t>(height);
  g.channels = static_cast<int32_t>(channels);
  g.border = border;
  g.border_value = border_value & 0xFF;
  g.ksize = k;
  g.arbitrary = fixed ? 0 : 1;
  g.vert_saturates = (!fixed && width * channels >= 16) ? 1 : 0;
  g.arb_border_len = static_cast<int32_t>((channels * r + 7) / 8 * 8);
  memcpy(g.half, half, r + 1);
  // Vertical result of a column inside a CONSTANT border: sum of all weights
  // times the border value, rounded like the vertical pass.
  const uint32_t acc = static_cast<uint32_t>(sum) * (border_value & 0xFF) + 128u;
  g.v_const = static_cast<int32_t>(g.vert_saturates ? (std::min(acc, 0xFFFFu) >> 8)
                                                    : ((acc >> 8) & 0xFFu));
  return KLEIDICV_OK;
}

kleidicv_error_t prepare_separable(int elem, const void *src, size_t src_stride, void *dst,
                                   size_t dst_stride, size_t width, size_t height,
                                   size_t channels, const void *kernel_x, size_t kernel_width,
                                   const void *kernel_y, size_t kernel_height, int border,
                                   bool ext, int border_value, Prepared *out) {
  const size_t es = elem == 1 ? 1 : 2;
  // separable_filter_2d_api.cpp:19-26, then the stripe checks
  // (separable_filter_2d_neon.cpp:229-235).
  if (kernel_width != 5 || kernel_height != 5) return KLEIDICV_ERROR_NOT_IMPLEMENTED;
  if (width < kernel_width - 1 || height < kernel_width - 1) return KLEIDICV_ERROR_NOT_IMPLEMENTED;
  if (!border_supported(border, ext)) return KLEIDICV_ERROR_NOT_IMPLEMENTED;
  if (!src) return KLEIDICV_ERROR_NULL_POINTER;
  if (stride_misaligned(src_stride, height, es)) return KLEIDICV_ERROR_ALIGNMENT;
  if (!dst) return KLEIDICV_ERROR_NULL_POINTER;
  if (stride_misaligned(dst_stride, height, es)) return KLEIDICV_ERROR_ALIGNMENT;
  if (!image_size_ok(width, height)) return KLEIDICV_ERROR_RANGE;
  if (!kernel_x || !kernel_y) return KLEIDICV_ERROR_NULL_POINTER;
  if (channels > kMaxChannels) return KLEIDICV_ERROR_NOT_IMPLEMENTED;
  if (!device_dims_ok(width * channels * es, height)) return KLEIDICV_ERROR_RANGE;

  *out = Prepared{};
  if (channels == 0) return KLEIDICV_OK;
  out->kind = Prepared::FUSED;
  FilterJob &j = out->fused;
  const int bv = elem == 1 ? (border_value & 0xFF) : (border_value & 0xFFFF);
  fill_common(j, src, src_stride, dst, dst_stride, width, height, channels, border, bv);
  j.ksize = 5;
  j.mode = elem == 1 ? MODE_SEP_U8 : (elem == 2 ? MODE_SEP_U16 : MODE_SEP_S16);
  for (int t = 0; t < 5; ++t) {
    if (elem == 1) {
      j.wx[t] = static_cast<const uint8_t *>(kernel_x)[t];
      j.wy[t] = static_cast<const uint8_t *>(kernel_y)[t];
    } else if (elem == 2) {
      j.wx[t] = static_cast<const uint16_t *>(kernel_x)[t];
      j.wy[t] = static_cast<const uint16_t *>(kernel_y)[t];
    } else {
      j.wx[t] = static_cast<const int16_t *>(kernel_x)[t];
      j.wy[t] = static_cast<const int16_t *>(kernel_y)[t];
    }
  }
  // Narrow taps: no intermediate sum can leave the accumulator width, so the
  // kernel may add without per-product saturation (identical results).
  //   u8:  every 16-bit lane sum <= 255 * sum(taps) <= 65535 in both passes;
  //   u16: every u32 sum <= 65535 * sum(taps) < 2^32 in both passes;
  //   s16: |vertical| <= 32768 * sum|ky| and |horizontal| <= 32768 *
  //        sum|kx| * sum|ky| < 2^31, so no saturating add ever saturates.
  long sx = 0, sy = 0;
  for (int t = 0; t < 5; ++t) {
    sx += j.wx[t] < 0 ? -static_cast<long>(j.wx[t]) : j.wx[t];
    sy += j.wy[t] < 0 ? -static_cast<long>(j.wy[t]) : j.wy[t];
  }
  if (elem == 1) j.narrow = sx <= 257 && sy <= 257;
  else if (elem == 2) j.narrow = sx <= 65537 && sy <= 65537;
  else j.narrow = sy <= 65535 && sx * sy <= 65535;
  return KLEIDICV_OK;
}

kleidicv_error_t prepare_blurdown(const uint8_t *src, size_t src_stride, size_t src_width,
                                  size_t src_height, uint8_t *dst, size_t dst_stride,
                                  size_t channels, int border, bool ext, int border_value,
                                  Prepared *out) {
  // blur_and_downsample_api.cpp:23-31, then blur_and_downsample_neon.cpp:322-324
  if (!(src_width >= 4 && src_height >= 4 && channels >= 1 && channels <= kMaxChannels))
    return KLEIDICV_ERROR_NOT_IMPLEMENTED;
  if (!border_supported(border, ext)) return KLEIDICV_ERROR_NOT_IMPLEMENTED;
  if (!src || !dst) return KLEIDICV_ERROR_NULL_POINTER;
  if (!image_size_ok(src_width, src_height)) return KLEIDICV_ERROR_RANGE;
  if (!device_dims_ok(src_width * channels, src_height)) return KLEIDICV_ERROR_RANGE;

  *out = Prepared{};
  out->kind = Prepared::FUSED;
  FilterJob &j = out->fused;
  fill_common(j, src, src_stride, dst, dst_stride, src_width, src_height, channels, border,
              border_value & 0xFF);
  j.out_width = static_cast<int32_t>((src_width + 1) / 2);
  j.out_height = static_cast<int32_t>((src_height + 1) / 2);
  j.mode = MODE_BLURDOWN;
  j.ksize = 5;
  for (int t = 0; t < 5; ++t) j.wy[t] = j.wx[t] = binomial_coef(5, t);
  return KLEIDICV_OK;
}

kleidicv_error_t prepare_sobel(bool horizontal, const uint8_t *src, size_t src_stride,
                               int16_t *dst, size_t dst_stride, size_t width, size_t height,
                               size_t channels, Prepared *out) {
  // sobel_api.cpp:22-31 (sobel_is_implemented, filters/sobel.h:30-33), then
  // the stripe checks of sobel_neon.cpp:135-141 (u8 source strides cannot be
  // misaligned).
  if (!(width >= 2 && height >= 2)) return KLEIDICV_ERROR_NOT_IMPLEMENTED;
  if (!src) return KLEIDICV_ERROR_NULL_POINTER;
  if (!dst) return KLEIDICV_ERROR_NULL_POINTER;
  if (stride_misaligned(dst_stride, height, 2)) return KLEIDICV_ERROR_ALIGNMENT;
  if (!image_size_ok(width, height)) return KLEIDICV_ERROR_RANGE;
  if (channels > kMaxChannels) return KLEIDICV_ERROR_NOT_IMPLEMENTED;
  if (!device_dims_ok(2 * width * channels, height)) return KLEIDICV_ERROR_RANGE;

  *out = Prepared{};
  if (channels == 0) return KLEIDICV_OK;
  out->kind = Prepared::FUSED;
  FilterJob &j = out->fused;
  // The only border of both derivatives is REPLICATE (sobel_neon.cpp:159,193).
  fill_common(j, src, src_stride, dst, dst_stride, width, height, channels, BORDER_REPLICATE, 0);
  j.ksize = 3;
  j.mode = horizontal ? MODE_SOBEL_X : MODE_SOBEL_Y;
  return KLEIDICV_OK;
}

// ---------------------------------------------------------------------------
// Tiling.
TileShape tile_shape_for(const FilterJob &j, int sm_count) {
  const int es = elem_size(j.mode);
  const long wcb = static_cast<long>(j.width) * j.channels * es;
  TileShape t{};
  // Autotuned shapes (committed table) win when present; a row with threads
  // 0 keeps the heuristic's warps per CTA below.
  const bool tuned = lookup_tile_shape(j.mode, j.ksize, j.channels, wcb, j.out_height, &t.threads,
                                       &t.tile_rows, &t.stage_rows, &t.stages);
  if (tuned && t.threads > 0) return t;
  const int hc = halo_chunks(j);
  const long chunks = (wcb + kChunk - 1) / kChunk;  // 16-byte chunks per source row
  const int wi = 32 - 2 * hc;                        // interior chunks per warp
  const int warps = static_cast<int>(std::min<long>(4, std::max<long>(1, (chunks + wi - 1) / wi)));
  t.threads = 32 * warps;
  if (tuned) return t;
  t.tile_rows = 0;  // chosen from the measured occupancy (finish_plan)
  t.stage_rows = 4;
  t.stages = 0;     // the ring depth rule's default
  return t;
}

// Ring depth rule.  A block of output rows reads block_in_rows consecutive
// source rows starting at a multiple of the block's row step; `need` is the
// most stages such a window can touch.  The ring holds need + 2 stages: the
// block's own plus two stages of copies in flight ahead of it.  With at least
// `need` stages a consumer warp never waits for a stage that cannot be issued
// until a warp behind it releases one.  stage_rows is a power of two; the
// ring has at most 16 stages (the mbarrier area), so large kernels get taller
// stages.
static void fix_ring(FilterJob &j) {
  auto pow2 = [](int v) {
    int p = 1;
    while (p < v) p <<= 1;
    return p;
  };
  const int in_rows = block_in_rows(j.mode, j.ksize);
  const int step = (j.mode == MODE_BLURDOWN ? 2 : 1) * block_out_rows(j.mode, j.ksize);
  int rb = std::max(1, std::min(pow2(j.stage_rows), 64));
  int ns = 0;
  for (;; rb <<= 1) {
    const int g = std::gcd(step, rb);
    int need = 1;
    for (int o = 0; o < rb; o += g) need = std::max(need, (o + in_rows - 1) / rb + 1);
    // Explicit stage counts (autotune table, tuning knob) need only the
    // safety minimum; the default keeps two stages of copies in flight.
    ns = j.stages > 0 ? std::max(j.stages, need) : need + 2;
    if (ns <= 16 || rb >= 64) break;
  }
  j.stage_rows = rb;
  j.stages = std::min(ns, 16);
}

void apply_tile_shape(FilterJob &j, const TileShape &t) {
  const int es = elem_size(j.mode);
  const long wcb = static_cast<long>(j.width) * j.channels * es;
  j.threads = t.threads;
  j.tile_rows = t.tile_rows;
  j.stage_rows = t.stage_rows;
  j.stages = t.stages;
  fix_ring(j);
  j.halo_chunks = halo_chunks(j);
  // Warps x interior chunks per warp.
  const int interior = (j.threads / 32) * (32 - 2 * j.halo_chunks);
  if (j.mode == MODE_BLURDOWN) {
    j.strip_out_bytes = interior * 8;
    j.strips = static_cast<int32_t>(
        (static_cast<long>(j.out_width) * j.channels + j.strip_out_bytes - 1) / j.strip_out_bytes);
  } else {
    j.strip_out_bytes = interior * kChunk;
    j.strips = static_cast<int32_t>((wcb + j.strip_out_bytes - 1) / j.strip_out_bytes);
  }
  j.row_tiles = j.tile_rows > 0 ? (j.out_height + j.tile_rows - 1) / j.tile_rows : 0;
}

// Bands when the tile shape left them open.  The resident CTAs of one wave
// (occupancy x SMs) each take one tile, and every SM should get the same
// work: the bands are whole blocks of output rows high, tile_rows or
// tile_rows + block_out_rows, so that strips x bands fills the wave exactly
// (a persistent CTA walks further tiles when there are more).
void finish_plan(FilterJob &j, int sm_count) {
  const int m = block_out_rows(j.mode, j.ksize);
  j.big_bands = 0;
  if (j.tile_rows <= 0) {
    const int occ = std::max(1, fused_blocks_per_sm(j));
    const long target = static_cast<long>(occ) * std::max(sm_count, 1);
    const long bands = std::max(1L, target / std::max<long>(j.strips, 1));
    const long q = m * (j.out_height / (bands * m));
    if (q == 0) {
      j.tile_rows = m;
      j.row_tiles = (j.out_height + m - 1) / m;
    } else {
      j.tile_rows = static_cast<int32_t>(q);
      j.row_tiles = static_cast<int32_t>(bands);
      j.big_bands = static_cast<int32_t>((j.out_height - bands * q) / m);
    }
    return;
  }
  j.row_tiles = (j.out_height + j.tile_rows - 1) / j.tile_rows;
}

void plan_fused(FilterJob &j, int sm_count) { apply_tile_shape(j, tile_shape_for(j, sm_count)); }

void encode_tma(FilterJob &j) {
  j.use_tma = 0;
  j.box_lbw = 8;
  const long wcb = static_cast<long>(j.width) * j.channels * elem_size(j.mode);
  if ((reinterpret_cast<uintptr_t>(j.src) & 15) != 0 || (j.src_stride & 15) != 0) return;
  if (wcb < 256 || j.height < 1 || j.stage_rows > 256) return;
  auto encode = tensor_map_encoder();
  if (!encode) return;
  // Rows that are a whole number of 8-byte units are viewed as u64 elements so
  // that one box spans 2048 bytes (one TMA per stage for a 4-warp strip).
  const bool wide = (wcb % 8) == 0;
  const cuuint64_t strides[1] = {static_cast<cuuint64_t>(j.src_stride)};
  const cuuint32_t estr[2] = {1u, 1u};
  auto enc = [&](CUtensorMap *m, bool w, cuuint32_t rows) {
    const cuuint64_t dims[2] = {static_cast<cuuint64_t>(w ? wcb / 8 : wcb),
                                static_cast<cuuint64_t>(j.height)};
    const cuuint32_t box[2] = {256u, rows};
    return encode(m, w ? CU_TENSOR_MAP_DATA_TYPE_UINT64 : CU_TENSOR_MAP_DATA_TYPE_UINT8, 2,
                  const_cast<uint8_t *>(j.src), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                  CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) ==
           CUDA_SUCCESS;
  };
  const cuuint32_t rb = static_cast<cuuint32_t>(j.stage_rows);
  if (!enc(&j.tmap, wide, rb) || !enc(&j.tmap_row, wide, 1u)) return;
  // The byte-unit wrap maps serve only a WRAP border (the far end of the row).
  if (j.border == BORDER_WRAP && (!enc(&j.tmap_wrap, false, rb) || !enc(&j.tmap_wrap_row, false, 1u)))
    return;
  j.box_lbw = wide ? 11 : 8;
  j.use_tma = 1;
}

// ---------------------------------------------------------------------------
// Context plumbing.
kleidicv_error_t cuda_status(kleidicv_gpu_context *ctx, cudaError_t e) {
  if (e == cudaSuccess) return KLEIDICV_OK;
  if (ctx) ctx->last_cuda_error = e;
  return KLEIDICV_GPU_ERROR_CUDA;
}

cudaError_t upload_async(kleidicv_gpu_context *ctx, void *dst, const void *src, size_t bytes) {
  if (bytes == 0) return cudaSuccess;
  std::lock_guard<std::mutex> lock(ctx->upload_mutex);
  kleidicv_gpu_context::UploadSlot &u = ctx->upload[ctx->upload_next];
  ctx->upload_next = (ctx->upload_next + 1) % kleidicv_gpu_context::kUploadSlots;
  cudaError_t e = u.done ? cudaEventSynchronize(u.done) : cudaEventCreateWithFlags(&u.done, cudaEventDisableTiming);
  if (e != cudaSuccess) return e;
  if (u.bytes < bytes) {
    if (u.host) cudaFreeHost(u.host);
    u.host = nullptr;
    u.bytes = 0;
    e = cudaHostAlloc(&u.host, bytes, cudaHostAllocPortable);
    if (e != cudaSuccess) {
      u.host = nullptr;
      return e;
    }
    u.bytes = bytes;
  }
  memcpy(u.host, src, bytes);
  e = cudaMemcpyAsync(dst, u.host, bytes, cudaMemcpyHostToDevice, ctx->stream);
  if (e != cudaSuccess) return e;
  return cudaEventRecord(u.done, ctx->stream);
}

void *ctx_alloc(kleidicv_gpu_context *ctx, size_t bytes) {
  int f = ctx->fail_allocs.load();
  while (f > 0) {
    if (ctx->fail_allocs.compare_exchange_weak(f, f - 1)) return nullptr;
  }
  if (ctx->pool_used.load() + bytes > ctx->pool_limit) return nullptr;
  void *p = nullptr;
  if (cudaMallocAsync(&p, bytes, ctx->stream) != cudaSuccess) return nullptr;
  ctx->pool_used += bytes;
  return p;
}

void ctx_free(kleidicv_gpu_context *ctx, void *p, size_t bytes) {
  if (!p) return;
  cudaFreeAsync(p, ctx->stream);
  ctx->pool_used -= bytes;
}

namespace {
thread_local kleidicv_gpu_context *t_default_ctx = nullptr;
}

kleidicv_error_t resolve_context(kleidicv_gpu_context *&ctx) {
  if (ctx) return KLEIDICV_OK;
  if (!t_default_ctx) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return KLEIDICV_GPU_ERROR_NO_DEVICE;
    kleidicv_error_t e = kleidicv_gpu_context_create(&t_default_ctx, dev, nullptr, 0);
    if (e != KLEIDICV_OK) return e;
  }
  ctx = t_default_ctx;
  return KLEIDICV_OK;
}

kleidicv_error_t execute(kleidicv_gpu_context *ctx, Prepared &p) {
  switch (p.kind) {
    case Prepared::NOTHING:
      return KLEIDICV_OK;
    case Prepared::COPY:
      return cuda_status(ctx, cudaMemcpy2DAsync(p.dst, p.dst_stride, p.src, p.src_stride,
                                                p.row_bytes, p.rows, cudaMemcpyDeviceToDevice,
                                                ctx->stream));
    case Prepared::FUSED: {
      if (p.fused.mode == MODE_BLURDOWN && ctx->tune_threads <= 0) {
        // One level: the tiled blur-and-downsample kernel of pyramid.cu.
        PyrLaunch L{};
        pyr_entry(L.inline_entries[0], p.fused.src, p.fused.src_stride, p.fused.dst, p.fused.dst_stride,
                  p.fused.width, p.fused.height, p.fused.channels, p.fused.border, p.fused.border_value,
                  pyramid_warps(p.fused.channels, ctx->sm_count));
        L.phase_begin[0] = 0;
        L.phase_begin[1] = 1;
        L.phases = 1;
        L.channels = p.fused.channels;
        L.barrier = reinterpret_cast<unsigned *>(ctx->d_err + 1);
        L.err_flag = ctx->d_err;
        ctx->launches += 1;
        return cuda_status(ctx, launch_pyramid(L, ctx->sm_count, ctx->stream));
      }
      if (ctx->tune_threads <= 0 && gauss8_eligible(p.fused)) {
        // Four-channel generated 3x3 / 5x5 / 7x7: the streaming kernel of gauss8.cu.
        ctx->launches += 1;
        return cuda_status(ctx, launch_gauss8(p.fused, ctx->sm_count, ctx->stream));
      }
      if (ctx->tune_threads <= 0 && sep16_eligible(p.fused)) {
        // One-channel 16-bit 5x5: the fp32 streaming kernel of sep16.cu.
        ctx->launches += 1;
        return cuda_status(ctx, launch_sep16(p.fused, ctx->sm_count, ctx->stream));
      }
      // A one-channel 16-bit call whose rows are not 16-byte aligned would take
      // the tiled kernel; from 1 MiB up its source is first copied into a pool
      // image with 16-byte rows so that the streaming kernel of sep16.cu takes
      // it (3841x2160 u16: 34 us against 44 us).  Other modes gain nothing from
      // the copy: the tiled kernel's loads and stores handle unaligned rows.
      if (ctx->tune_threads <= 0) {
        FilterJob probe = p.fused;
        const long wcb = static_cast<long>(p.fused.width) * p.fused.channels * elem_size(p.fused.mode);
        const size_t stride = (static_cast<size_t>(wcb) + 15) / 16 * 16;
        probe.src = reinterpret_cast<const uint8_t *>(uintptr_t{256});  // any 16-byte aligned base
        probe.src_stride = static_cast<int64_t>(stride);
        if (static_cast<size_t>(wcb) * p.fused.height >= (size_t{1} << 20) && sep16_eligible(probe)) {
          const size_t bytes = stride * p.fused.height;
          uint8_t *realigned = static_cast<uint8_t *>(ctx_alloc(ctx, bytes));
          if (realigned) {
            cudaError_t e = launch_realign(p.fused.src, p.fused.src_stride, realigned, static_cast<int64_t>(stride),
                                           wcb, p.fused.height, ctx->sm_count, ctx->stream);
            if (e == cudaSuccess) {
              p.fused.src = realigned;
              p.fused.src_stride = static_cast<int64_t>(stride);
              e = launch_sep16(p.fused, ctx->sm_count, ctx->stream);
            }
            ctx->launches += 2;
            // Stream-ordered: the copy is released after the filter has read it.
            ctx_free(ctx, realigned, bytes);
            return cuda_status(ctx, e);
          }
        }
      }
      if (ctx->tune_threads > 0) {
        TileShape t{ctx->tune_threads, ctx->tune_tile_rows, ctx->tune_stage_rows, ctx->tune_stages};
        apply_tile_shape(p.fused, t);
      } else {
        plan_fused(p.fused, ctx->sm_count);
      }
      encode_tma(p.fused);
      finish_plan(p.fused, ctx->sm_count);
      cudaError_t e = launch_fused(p.fused, ctx->d_err, ctx->stream);
      ctx->launches += 1;
      return cuda_status(ctx, e);
    }
    case Prepared::GENERIC: {
      const GenericJob &g = p.generic;
      const size_t vstride = (static_cast<size_t>(g.width) * g.channels + 15) / 16 * 16;
      const size_t bytes = vstride * g.height;
      uint8_t *scratch = static_cast<uint8_t *>(ctx_alloc(ctx, bytes));
      if (!scratch) return KLEIDICV_ERROR_ALLOCATION;
      cudaError_t e = launch_generic_gaussian(g, scratch, vstride, ctx->stream);
      ctx->launches += 2;
      ctx_free(ctx, scratch, bytes);
      return cuda_status(ctx, e);
    }
  }
  return KLEIDICV_OK;
}

}  // namespace kcv

// ===========================================================================
// C ABI
using namespace kcv;

extern "C" {

kleidicv_error_t kleidicv_gpu_context_create(kleidicv_gpu_context_t **out, int device,
                                             void *stream, size_t pool_limit_bytes) {
  if (!out) return KLEIDICV_ERROR_NULL_POINTER;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count)
    return KLEIDICV_GPU_ERROR_NO_DEVICE;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return KLEIDICV_GPU_ERROR_NO_DEVICE;
  if (prop.major != 10 || prop.minor != 3) return KLEIDICV_GPU_ERROR_NO_DEVICE;  // sm_103 only
  DeviceGuard guard(device);
  auto *ctx = new kleidicv_gpu_context();
  ctx->device = device;
  ctx->stream = static_cast<cudaStream_t>(stream);
  ctx->pool_limit = pool_limit_bytes ? pool_limit_bytes : (40ull << 30);
  ctx->sm_count = prop.multiProcessorCount;
  // d_err[0]: the device error flag; d_err[1]: the pyramid kernel's grid
  // barrier counter.
  if (cudaMalloc(&ctx->d_err, 4 * sizeof(int)) != cudaSuccess ||
      cudaMemset(ctx->d_err, 0, 4 * sizeof(int)) != cudaSuccess) {
    delete ctx;
    return KLEIDICV_GPU_ERROR_CUDA;
  }
  *out = ctx;
  return KLEIDICV_OK;
}

kleidicv_error_t kleidicv_gpu_context_destroy(kleidicv_gpu_context_t *ctx) {
  if (!ctx) return KLEIDICV_ERROR_NULL_POINTER;
  DeviceGuard guard(ctx->device);
  shutdown_async(ctx);
  cudaStreamSynchronize(ctx->stream);
  for (cudaStream_t s : ctx->branches) {
    cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
  }
  for (cudaEvent_t e : ctx->branch_events) cudaEventDestroy(e);
  if (ctx->fork_event) cudaEventDestroy(ctx->fork_event);
  if (ctx->pinned) cudaFreeHost(ctx->pinned);
  for (auto &u : ctx->upload) {
    if (u.host) cudaFreeHost(u.host);
    if (u.done) cudaEventDestroy(u.done);
  }
  cudaFree(ctx->d_err);
  delete ctx;
  return KLEIDICV_OK;
}

kleidicv_error_t kleidicv_gpu_context_set_stream(kleidicv_gpu_context_t *ctx, void *stream) {
  if (!ctx) return KLEIDICV_ERROR_NULL_POINTER;
  ctx->stream = static_cast<cudaStream_t>(stream);
  return KLEIDICV_OK;
}

void *kleidicv_gpu_context_get_stream(const kleidicv_gpu_context_t *ctx) {
  return ctx ? static_cast<void *>(ctx->stream) : nullptr;
}

kleidicv_error_t kleidicv_gpu_context_synchronize(kleidicv_gpu_context_t *ctx) {
  if (resolve_context(ctx) != KLEIDICV_OK) return KLEIDICV_GPU_ERROR_NO_DEVICE;
  DeviceGuard guard(ctx->device);
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_status(ctx, e);
  int flag = 0;
  e = cudaMemcpy(&flag, ctx->d_err, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_status(ctx, e);
  if (flag) {
    cudaMemset(ctx->d_err, 0, sizeof(int));
    return KLEIDICV_GPU_ERROR_TIMEOUT;
  }
  if (ctx->last_cuda_error != cudaSuccess) {
    ctx->last_cuda_error = cudaSuccess;
    return KLEIDICV_GPU_ERROR_CUDA;
  }
  return KLEIDICV_OK;
}

void kleidicv_gpu_context_fail_next_allocations(kleidicv_gpu_context_t *ctx, int count) {
  if (ctx) ctx->fail_allocs = count;
}

uint64_t kleidicv_gpu_context_launch_count(const kleidicv_gpu_context_t *ctx) {
  return ctx ? ctx->launches.load() : 0;
}

kleidicv_error_t kleidicv_gpu_context_set_tile_shape(kleidicv_gpu_context_t *ctx, int threads,
                                                     int tile_rows, int stage_rows, int stages) {
  if (!ctx) return KLEIDICV_ERROR_NULL_POINTER;
  if (threads != 0 && (threads % 32 != 0 || threads < 32 || threads > 128 || tile_rows < 0 ||
                       stage_rows < 1 || stages < 0 || stages > 16))
    return KLEIDICV_ERROR_RANGE;
  ctx->tune_threads = threads;
  ctx->tune_tile_rows = tile_rows;
  ctx->tune_stage_rows = stage_rows;
  ctx->tune_stages = stages;
  return KLEIDICV_OK;
}

static kleidicv_error_t run(kleidicv_gpu_context_t *ctx, kleidicv_error_t prep, Prepared &p) {
  if (prep != KLEIDICV_OK) return prep;
  if (p.kind == Prepared::NOTHING) return KLEIDICV_OK;
  kleidicv_error_t e = resolve_context(ctx);
  if (e != KLEIDICV_OK) return e;
  DeviceGuard guard(ctx->device);
  return execute(ctx, p);
}

kleidicv_error_t kleidicv_gpu_gaussian_blur_u8(const uint8_t *src, size_t src_stride, uint8_t *dst,
                                               size_t dst_stride, size_t width, size_t height,
                                               size_t channels, size_t kernel_width,
                                               size_t kernel_height, float sigma_x,
                                               float sigma_y, kleidicv_border_type_t border_type,
                                               kleidicv_gpu_context_t *ctx) {
  Prepared p;
  auto e = prepare_gaussian(src, src_stride, dst, dst_stride, width, height, channels,
                            kernel_width, kernel_height, sigma_x, sigma_y, border_type, false, 0,
                            &p);
  return run(ctx, e, p);
}

kleidicv_error_t kleidicv_gpu_gaussian_blur_u8_ex(
    const uint8_t *src, size_t src_stride, uint8_t *dst, size_t dst_stride, size_t width,
    size_t height, size_t channels, size_t kernel_width, size_t kernel_height, float sigma_x,
    float sigma_y, kleidicv_border_type_t border_type, uint8_t border_value,
    kleidicv_gpu_context_t *ctx) {
  Prepared p;
  auto e = prepare_gaussian(src, src_stride, dst, dst_stride, width, height, channels,
                            kernel_width, kernel_height, sigma_x, sigma_y, border_type, true,
                            border_value, &p);
  return run(ctx, e, p);
}

kleidicv_error_t kleidicv_gpu_separable_filter_2d_u8(
    const uint8_t *src, size_t src_stride, uint8_t *dst, size_t dst_stride, size_t width,
    size_t height, size_t channels, const uint8_t *kernel_x, size_t kernel_width,
    const uint8_t *kernel_y, size_t kernel_height, kleidicv_border_type_t border_type,
    kleidicv_gpu_context_t *ctx) {
  Prepared p;
  auto e = prepare_separable(1, src, src_stride, dst, dst_stride, width, height, channels,
                             kernel_x, kernel_width, kernel_y, kernel_height, border_type, false,
                             0, &p);
  return run(ctx, e, p);
}

kleidicv_error_t kleidicv_gpu_separable_filter_2d_u16(
    const uint16_t *src, size_t src_stride, uint16_t *dst, size_t dst_stride, size_t width,
    size_t height, size_t channels, const uint16_t *kernel_x, size_t kernel_width,
    const uint16_t *kernel_y, size_t kernel_height, kleidicv_border_type_t border_type,
    kleidicv_gpu_context_t *ctx) {
  Prepared p;
  auto e = prepare_separable(2, src, src_stride, dst, dst_stride, width, height, channels,
                             kernel_x, kernel_width, kernel_y, kernel_height, border_type, false,
                             0, &p);
  return run(ctx, e, p);
}

kleidicv_error_t kleidicv_gpu_separable_filter_2d_u8_ex(
    const uint8_t *src, size_t src_stride, uint8_t *dst, size_t dst_stride, size_t width,
    size_t height, size_t channels, const uint8_t *kernel_x, size_t kernel_width,
    const uint8_t *kernel_y, size_t kernel_height, kleidicv_border_type_t border_type,
    uint8_t border_value, kleidicv_gpu_context_t *ctx) {
  Prepared p;
  auto e = prepare_separable(1, src, src_stride, dst, dst_stride, width, height, channels,
                             kernel_x, kernel_width, kernel_y, kernel_height, border_type, true,
                             border_value, &p);
  return run(ctx, e, p);
}

kleidicv_error_t kleidicv_gpu_separable_filter_2d_u16_ex(
    const uint16_t *src, size_t src_stride, uint16_t *dst, size_t dst_stride, size_t width,
    size_t height, size_t channels, const uint16_t *kernel_x, size_t kernel_width,
    const uint16_t *kernel_y, size_t kernel_height, kleidicv_border_type_t border_type,
    uint16_t border_value, kleidicv_gpu_context_t *ctx) {
  Prepared p;
  auto e = prepare_separable(2, src, src_stride, dst, dst_stride, width, height, channels,
                             kernel_x, kernel_width, kernel_y, kernel_height, border_type, true,
                             border_value, &p);
  return run(ctx, e, p);
}

kleidicv_error_t kleidicv_gpu_separable_filter_2d_s16_ex(
    const int16_t *src, size_t src_stride, int16_t *dst, size_t dst_stride, size_t width,
    size_t height, size_t channels, const int16_t *kernel_x, size_t kernel_width,
    const int16_t *kernel_y, size_t kernel_height, kleidicv_border_type_t border_type,
    int16_t border_value, kleidicv_gpu_context_t *ctx) {
  Prepared p;
  auto e = prepare_separable(3, src, src_stride, dst, dst_stride, width, height, channels,
                             kernel_x, kernel_width, kernel_y, kernel_height, border_type, true,
                             static_cast<uint16_t>(border_value), &p);
  return run(ctx, e, p);
}

kleidicv_error_t kleidicv_gpu_blur_and_downsample_u8(const uint8_t *src, size_t src_stride,
                                                     size_t src_width, size_t src_height,
                                                     uint8_t *dst, size_t dst_stride,
                                                     size_t channels,
                                                     kleidicv_border_type_t border_type,
                                                     kleidicv_gpu_context_t *ctx) {
  Prepared p;
  auto e = prepare_blurdown(src, src_stride, src_width, src_height, dst, dst_stride, channels,
                            border_type, false, 0, &p);
  return run(ctx, e, p);
}

kleidicv_error_t kleidicv_gpu_blur_and_downsample_u8_ex(
    const uint8_t *src, size_t src_stride, size_t src_width, size_t src_height, uint8_t *dst,
    size_t dst_stride, size_t channels, kleidicv_border_type_t border_type, uint8_t border_value,
    kleidicv_gpu_context_t *ctx) {
  Prepared p;
  auto e = prepare_blurdown(src, src_stride, src_width, src_height, dst, dst_stride, channels,
                            border_type, true, border_value, &p);
  return run(ctx, e, p);
}

kleidicv_error_t kleidicv_gpu_sobel_3x3_horizontal_s16_u8(const uint8_t *src, size_t src_stride,
                                                         int16_t *dst, size_t dst_stride,
                                                         size_t width, size_t height,
                                                         size_t channels,
                                                         kleidicv_gpu_context_t *ctx) {
  Prepared p;
  auto e = prepare_sobel(true, src, src_stride, dst, dst_stride, width, height, channels, &p);
  return run(ctx, e, p);
}

kleidicv_error_t kleidicv_gpu_sobel_3x3_vertical_s16_u8(const uint8_t *src, size_t src_stride,
                                                       int16_t *dst, size_t dst_stride,
                                                       size_t width, size_t height,
                                                       size_t channels,
                                                       kleidicv_gpu_context_t *ctx) {
  Prepared p;
  auto e = prepare_sobel(false, src, src_stride, dst, dst_stride, width, height, channels, &p);
  return run(ctx, e, p);
}

kleidicv_error_t kleidicv_gpu_build_pyramid_u8(const uint8_t *src, size_t src_stride,
                                               size_t src_width, size_t src_height,
                                               size_t channels, size_t levels,
                                               uint8_t *const *dst, const size_t *dst_strides,
                                               kleidicv_border_type_t border_type,
                                               kleidicv_gpu_context_t *ctx) {
  if (levels == 0) return KLEIDICV_OK;
  if (!dst || !dst_strides) return KLEIDICV_ERROR_NULL_POINTER;
  Prepared p[64];
  if (levels > 64) return KLEIDICV_ERROR_RANGE;
  const uint8_t *s = src;
  size_t ss = src_stride, w = src_width, h = src_height;
  for (size_t l = 0; l < levels; ++l) {
    kleidicv_error_t e = prepare_blurdown(s, ss, w, h, dst[l], dst_strides[l], channels,
                                          border_type, false, 0, &p[l]);
    if (e != KLEIDICV_OK) return e;
    s = dst[l];
    ss = dst_strides[l];
    w = (w + 1) / 2;
    h = (h + 1) / 2;
  }
  kleidicv_error_t e = resolve_context(ctx);
  if (e != KLEIDICV_OK) return e;
  DeviceGuard guard(ctx->device);
  if (ctx->tune_threads > 0) {  // a forced tile shape: the tiled stencil, one launch per level
    for (size_t l = 0; l < levels; ++l) {
      e = execute(ctx, p[l]);
      if (e != KLEIDICV_OK) return e;
    }
    return KLEIDICV_OK;
  }
  // Up to kPyrInline levels per launch, one phase per level.
  for (size_t l0 = 0; l0 < levels; l0 += kPyrInline) {
    const size_t n = std::min<size_t>(kPyrInline, levels - l0);
    PyrLaunch L{};
    for (size_t k = 0; k < n; ++k) {
      const FilterJob &j = p[l0 + k].fused;
      pyr_entry(L.inline_entries[k], j.src, j.src_stride, j.dst, j.dst_stride, j.width, j.height,
                static_cast<int>(channels), j.border, 0, pyramid_warps(static_cast<int>(channels), ctx->sm_count));
      L.phase_begin[k] = static_cast<int32_t>(k);
    }
    L.phase_begin[n] = static_cast<int32_t>(n);
    L.phases = static_cast<int32_t>(n);
    L.channels = static_cast<int32_t>(channels);
    L.barrier = reinterpret_cast<unsigned *>(ctx->d_err + 1);
    L.err_flag = ctx->d_err;
    ctx->launches += 1;
    e = cuda_status(ctx, launch_pyramid(L, ctx->sm_count, ctx->stream));
    if (e != KLEIDICV_OK) return e;
  }
  return KLEIDICV_OK;
}

kleidicv_error_t kleidicv_gpu_build_pyramids_u8(const kleidicv_gpu_pyramid_t *pyramids, size_t count,
                                                kleidicv_error_t *statuses, kleidicv_gpu_context_t *ctx) {
  if (count == 0) return KLEIDICV_OK;
  if (!pyramids) return KLEIDICV_ERROR_NULL_POINTER;
  // Validate every level of every pyramid first, as the single call does.
  std::vector<std::vector<Prepared>> prep(count);
  kleidicv_error_t first = KLEIDICV_OK;
  for (size_t i = 0; i < count; ++i) {
    const kleidicv_gpu_pyramid_t &py = pyramids[i];
    kleidicv_error_t e = KLEIDICV_OK;
    if (py.levels > 0 && (!py.dst || !py.dst_strides)) e = KLEIDICV_ERROR_NULL_POINTER;
    if (py.levels > static_cast<size_t>(kPyrMaxPhases)) e = KLEIDICV_ERROR_RANGE;
    const uint8_t *s = py.src;
    size_t ss = py.src_stride, w = py.src_width, h = py.src_height;
    for (size_t l = 0; e == KLEIDICV_OK && l < py.levels; ++l) {
      prep[i].emplace_back();
      e = prepare_blurdown(s, ss, w, h, py.dst[l], py.dst_strides[l], py.channels, py.border_type, false, 0,
                           &prep[i].back());
      s = py.dst[l];
      ss = py.dst_strides[l];
      w = (w + 1) / 2;
      h = (h + 1) / 2;
    }
    if (statuses) statuses[i] = e;
    if (e != KLEIDICV_OK && first == KLEIDICV_OK) first = e;
  }
  if (first != KLEIDICV_OK) return first;
  kleidicv_error_t e = resolve_context(ctx);
  if (e != KLEIDICV_OK) return e;
  DeviceGuard guard(ctx->device);
  // One launch per channel count: phase l holds level l + 1 of every image.
  for (int c = 1; c <= static_cast<int>(kMaxChannels); ++c) {
    std::vector<PyrEntry> entries;
    PyrLaunch L{};
    size_t phases = 0;
    for (size_t i = 0; i < count; ++i)
      if (static_cast<int>(pyramids[i].channels) == c) phases = std::max(phases, pyramids[i].levels);
    if (phases == 0) continue;
    const int warps = pyramid_warps(c, ctx->sm_count);
    for (size_t l = 0; l < phases; ++l) {
      L.phase_begin[l] = static_cast<int32_t>(entries.size());
      // The phase's images share the resident warps: each entry's bands are
      // sized for its share.
      int in_phase = 0;
      for (size_t i = 0; i < count; ++i)
        if (static_cast<int>(pyramids[i].channels) == c && l < pyramids[i].levels) ++in_phase;
      const int share = std::max(1, warps / std::max(in_phase, 1));
      int32_t items = 0;
      for (size_t i = 0; i < count; ++i) {
        if (static_cast<int>(pyramids[i].channels) != c || l >= pyramids[i].levels) continue;
        const FilterJob &j = prep[i][l].fused;
        PyrEntry en;
        pyr_entry(en, j.src, j.src_stride, j.dst, j.dst_stride, j.width, j.height, c, j.border, 0, share);
        items += en.item_end;
        en.item_end = items;
        entries.push_back(en);
      }
    }
    L.phase_begin[phases] = static_cast<int32_t>(entries.size());
    L.phases = static_cast<int32_t>(phases);
    L.channels = c;
    L.barrier = reinterpret_cast<unsigned *>(ctx->d_err + 1);
    L.err_flag = ctx->d_err;
    const size_t bytes = entries.size() * sizeof(PyrEntry);
    PyrEntry *table = nullptr;
    if (entries.size() <= static_cast<size_t>(kPyrInline)) {
      std::copy(entries.begin(), entries.end(), L.inline_entries);
    } else {
      table = static_cast<PyrEntry *>(ctx_alloc(ctx, bytes));
      if (!table) return KLEIDICV_ERROR_ALLOCATION;
      cudaError_t ce = upload_async(ctx, table, entries.data(), bytes);
      if (ce != cudaSuccess) {
        ctx_free(ctx, table, bytes);
        return cuda_status(ctx, ce);
      }
      L.entries = table;
    }
    ctx->launches += 1;
    e = cuda_status(ctx, launch_pyramid(L, ctx->sm_count, ctx->stream));
    if (table) ctx_free(ctx, table, bytes);
    if (e != KLEIDICV_OK) return e;
  }
  return KLEIDICV_OK;
}

}  // extern "C"
