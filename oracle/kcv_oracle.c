/*
 * CPU oracle for KleidiCV's separable-filter hot path.  TEST INFRASTRUCTURE
 * ONLY -- see kcv_oracle.h for the list of reference files restated here and
 * for who may call this code.
 *
 * The restatement follows the reference's *results*, not its vector code:
 * every output element is computed from the integer formula the NEON/SVE
 * classes implement (vertical pass first into the reference's intermediate
 * width, then the horizontal pass, then the reference's rounding or
 * saturation).  Rows are processed exactly like
 * SeparableFilterWorkspace::process (workspace/separable.h:112-141): one
 * widened intermediate row per output row.
 */
#include "kcv_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define KO_MAX_IMAGE_PIXELS ((1ULL << 48) - 1ULL) /* kleidicv.h:103 */
#define KO_MAX_CHANNELS 4                         /* kleidicv.h:110 */

/* ------------------------------------------------------------------------ */
/* Gaussian half kernel: restates kleidicv/include/kleidicv/filters/sigma.h:27-79
 * step by step in float arithmetic (this file is built with
 * -ffp-contract=off so no FMA contraction alters the float rounding). */
int ko_gaussian_half_kernel(uint8_t *half_kernel, size_t half_size,
                            float sigma) {
  const size_t mid = half_size - 1;
  const size_t ksize = mid * 2 + 1;
  if (sigma == 0.0f) {
    sigma = (float)ksize * 0.15f + 0.35f;
  }
  float gauss[255];
  const float coef = 1.0f / -(2.0f * sigma * sigma);
  float sum = 0.0f;
  for (size_t i = 0; i < mid; ++i) {
    const float d = (float)(mid - i);
    gauss[i] = expf(d * d * coef);
    sum += gauss[i];
  }
  const float scale = 256.0f / (sum * 2.0f + 1.0f);
  float carried = 0.0f;
  for (size_t i = 0; i < mid; ++i) {
    const float want = gauss[i] * scale - carried;
    const float got = roundf(want);
    half_kernel[i] = (uint8_t)got;
    carried = got - want;
  }
  const unsigned centre = (unsigned)(uint16_t)roundf(scale - carried);
  if (centre == 256u) {
    return 0;
  }
  half_kernel[mid] = (uint8_t)centre;
  return 1;
}

/* ------------------------------------------------------------------------ */
/* Border index map.  The reference's FixedBorderInfo<K> tables
 * (workspace/border_*.h) are single-fold mirrors/wraps that are exact as long
 * as n >= K - 1, which gaussian_blur_is_implemented and
 * separable_filter_2d_is_implemented guarantee.  The arbitrary-size path
 * (border_generic_neon.h:49-53,111-115) clamps, i.e. REPLICATE. */
long ko_border_map(long i, long n, int border) {
  if (i >= 0 && i < n) return i;
  switch (border) {
    case KO_BORDER_REPLICATE:
      return i < 0 ? 0 : n - 1;
    case KO_BORDER_REFLECT:
      return i < 0 ? -i - 1 : 2 * n - i - 1;
    case KO_BORDER_WRAP:
      return i < 0 ? i + n : i - n;
    case KO_BORDER_REVERSE:
      return i < 0 ? -i : 2 * n - i - 2;
    default: /* CONSTANT */
      return -1;
  }
}

/* ------------------------------------------------------------------------ */
enum { M_BINOM, M_SIGMA, M_SEP_U8, M_SEP_U16, M_SEP_S16, M_BLURDOWN, M_SOBEL_X, M_SOBEL_Y };

typedef struct {
  int mode;
  int ksize;
  int64_t wy[256]; /* vertical taps */
  int64_t wx[256]; /* horizontal taps */
  int shift;       /* binomial rounding shift */
  int border;
  int64_t border_value;
  int arbitrary;      /* odd sizes 11..255 other than 15/21 */
  int vert_saturates; /* arbitrary path: vertical pass ran on vectors */
  size_t arb_border_len; /* arbitrary path: elements per side handled by the
                            border vector paths (multiple of 8) */
  size_t width, height, channels; /* source geometry (pixels) */
  size_t out_width, out_height;
  const uint8_t *src;
  size_t src_stride;
  uint8_t *dst;
  size_t dst_stride;
  size_t elem_size;
} ko_job;

static int64_t load_elem(const ko_job *j, long row, long elem) {
  const uint8_t *p = j->src + (size_t)row * j->src_stride;
  switch (j->elem_size) {
    case 1:
      return p[elem];
    case 2:
      if (j->mode == M_SEP_S16) return ((const int16_t *)p)[elem];
      return ((const uint16_t *)p)[elem];
  }
  return 0;
}

static void store_elem(const ko_job *j, long row, long elem, int64_t v) {
  uint8_t *p = j->dst + (size_t)row * j->dst_stride;
  if (j->mode == M_SOBEL_X || j->mode == M_SOBEL_Y) {
    ((int16_t *)p)[elem] = (int16_t)v; /* u8 source, s16 destination */
  } else if (j->elem_size == 1) {
    p[elem] = (uint8_t)v;
  } else if (j->mode == M_SEP_S16) {
    ((int16_t *)p)[elem] = (int16_t)v;
  } else {
    ((uint16_t *)p)[elem] = (uint16_t)v;
  }
}

static int64_t sat_s32(int64_t v) {
  if (v > INT32_MAX) return INT32_MAX;
  if (v < INT32_MIN) return INT32_MIN;
  return v;
}

/* Vertical pass for one element position given the K source values. */
static int64_t vertical(const ko_job *j, const int64_t *s) {
  const int k = j->ksize;
  int64_t acc = 0;
  switch (j->mode) {
    case M_BINOM:
    case M_BLURDOWN:
      /* u16 row buffer, exact (gaussian_blur_fixed_neon.cpp:33-459). */
      for (int t = 0; t < k; ++t) acc += j->wy[t] * s[t];
      return acc;
    case M_SIGMA:
      /* u8 row buffer.  The weights sum to 256 almost everywhere, and then
       * (sum + 128) >> 8 fits 8 bits.  For the few (size, sigma) pairs whose
       * rounded weights sum to 257 the 16-bit accumulator can reach 65535:
       *  - fixed sizes: the vector path starts from 128 and wraps
       *    (gaussian_blur_fixed_neon.cpp:501-526), the scalar path wraps in
       *    uint16_t (:477-488); both give ((sum + 128) >> 8) mod 256;
       *  - arbitrary sizes: the vector path adds 128 with vqaddq, i.e.
       *    saturates (gaussian_blur_arbitrary_neon.cpp:193-194); it is used
       *    for every element when width*channels >= 16 (LoopUnroll2 with
       *    TryToAvoidTailLoop, utils.h:298-322), else the u32 scalar path
       *    (:232-244) wraps on the cast to uint8_t. */
      for (int t = 0; t < k; ++t) acc += j->wy[t] * s[t];
      if (j->arbitrary && j->vert_saturates)
        return (acc + 128 > 0xFFFF ? 0xFFFF : acc + 128) >> 8;
      return ((acc + 128) >> 8) & 0xFF;
    case M_SEP_U8:
      /* Saturating u16 accumulation (separable_filter_2d_neon.cpp:38-56). */
      for (int t = 0; t < k; ++t) acc += j->wy[t] * s[t];
      return acc > 0xFFFF ? 0xFFFF : acc;
    case M_SEP_U16:
      /* Saturating u32 accumulation (separable_filter_2d_neon.cpp:140-158). */
      for (int t = 0; t < k; ++t) acc += j->wy[t] * s[t];
      return acc > 0xFFFFFFFFLL ? 0xFFFFFFFFLL : acc;
    case M_SOBEL_X:
    case M_SOBEL_Y:
      /* s16 row buffer: [1 2 1] or [-1 0 1] (sobel_neon.cpp:36-53, 95-109);
       * |sum| <= 1020, so the reference's narrowing never wraps. */
      for (int t = 0; t < k; ++t) acc += j->wy[t] * s[t];
      return acc;
    case M_SEP_S16:
      /* Extension: product of tap 0, then saturating s32 adds in tap order. */
      acc = j->wy[0] * s[0];
      for (int t = 1; t < k; ++t) acc = sat_s32(acc + j->wy[t] * s[t]);
      return acc;
  }
  return 0;
}

/* Arbitrary-size horizontal pass (gaussian_blur_arbitrary_neon.cpp:81-124):
 * elements in the first and last `arb_border_len` positions go through the
 * border vector paths, whose vrshrn narrows (wraps); the middle span goes
 * through the vqaddq vector path (saturates) when it holds at least one full
 * 16-lane vector, else through the u32 scalar path (wraps). */
static int arbitrary_h_saturates(const ko_job *j, long x) {
  const long wc = (long)(j->width * j->channels);
  const long bl = (long)j->arb_border_len;
  if (wc <= 2 * bl) return 0;
  if (x < bl || x >= wc - bl) return 0;
  return wc - 2 * bl >= 16;
}

/* Arbitrary-size right border (gaussian_blur_arbitrary_neon.cpp:346-377,
 * border_generic_neon.h:80-98).  The last `arb_border_len` elements of a row
 * are computed by 8-lane vectors starting at width*channels - arb_border_len.
 * For the right-hand tap at distance d (columns) the vector starting at xv
 * reads elements xv + c*d .. +7; when all of them lie past the row end, the
 * reference builds the replicated lanes from an index pattern that, for
 * q = (xv + c*d - width*c) % c != 0, gives lanes 8-q..7 channel lane+c-8 of
 * the last pixel instead of channel (q+lane) % c.  Returns that channel for
 * output element e and tap distance d, or -1 where the lane is exact. */
static long arb_right_lane_channel(const ko_job *j, long e, long d) {
  const long c = (long)j->channels;
  const long wc = (long)j->width * c;
  const long bl = (long)j->arb_border_len;
  if (c == 1 || e < wc - bl) return -1;
  const long xv = wc - bl + (e - (wc - bl)) / 8 * 8;
  const long lane = e - xv;
  const long start = xv + c * d;
  if (start < wc) return -1;
  const long q = (start - wc) % c;
  if (q == 0 || lane < 8 - q) return -1;
  return lane + c - 8;
}

/* Horizontal pass for one output element given the K intermediate values. */
static int64_t horizontal(const ko_job *j, const int64_t *v, long x) {
  const int k = j->ksize;
  int64_t acc = 0;
  for (int t = 0; t < k; ++t) acc += j->wx[t] * v[t];
  switch (j->mode) {
    case M_BINOM:
      return (acc + (1LL << (j->shift - 1))) >> j->shift;
    case M_BLURDOWN:
      return (acc + 128) >> 8;
    case M_SIGMA:
      if (j->arbitrary && arbitrary_h_saturates(j, x))
        return (acc + 128 > 0xFFFF ? 0xFFFF : acc + 128) >> 8;
      return ((acc + 128) >> 8) & 0xFF;
    case M_SEP_U8:
      return acc > 0xFF ? 0xFF : acc;
    case M_SEP_U16:
      return acc > 0xFFFF ? 0xFFFF : acc;
    case M_SOBEL_X:
    case M_SOBEL_Y:
      /* [-1 0 1] or [1 2 1] of the row buffer (sobel_neon.cpp:58-69,
       * 114-127); |result| <= 1020. */
      return acc;
    case M_SEP_S16:
      if (acc > INT16_MAX) return INT16_MAX;
      if (acc < INT16_MIN) return INT16_MIN;
      return acc;
  }
  return 0;
}

/* Processes output rows [y0, y1).  For each output row the intermediate row
 * is computed over the whole source width (like the reference's widened row
 * buffer), then the horizontal pass reads it through the border map. */
static void run_rows(const ko_job *j, size_t y0, size_t y1, int64_t *vrow) {
  const long r = j->ksize / 2;
  const long w = (long)j->width, h = (long)j->height, c = (long)j->channels;
  const int step = j->mode == M_BLURDOWN ? 2 : 1;
  int64_t s[256], v[256];
  /* Intermediate value of a column that lies entirely in a CONSTANT border. */
  for (long t = 0; t < j->ksize; ++t) s[t] = j->border_value;
  const int64_t v_const = vertical(j, s);

  for (size_t oy = y0; oy < y1; ++oy) {
    const long y = (long)oy * step;
    for (long x = 0; x < w * c; ++x) {
      for (long t = 0; t < j->ksize; ++t) {
        const long ry = ko_border_map(y + t - r, h, j->border);
        s[t] = ry < 0 ? j->border_value : load_elem(j, ry, x);
      }
      vrow[x] = vertical(j, s);
    }
    for (long ox = 0; ox < (long)j->out_width; ++ox) {
      const long col = ox * step;
      for (long ch = 0; ch < c; ++ch) {
        for (long t = 0; t < j->ksize; ++t) {
          const long rc = ko_border_map(col + t - r, w, j->border);
          v[t] = rc < 0 ? v_const : vrow[rc * c + ch];
        }
        if (j->arbitrary) {
          for (long d = 1; d <= r; ++d) {
            const long qc = arb_right_lane_channel(j, ox * c + ch, d);
            if (qc >= 0) v[r + d] = vrow[(w - 1) * c + qc];
          }
        }
        store_elem(j, (long)oy, ox * c + ch, horizontal(j, v, ox * c + ch));
      }
    }
  }
}

typedef struct {
  const ko_job *job;
  size_t y0, y1;
  int failed;
} ko_stripe;

static void *stripe_main(void *arg) {
  ko_stripe *st = (ko_stripe *)arg;
  int64_t *vrow = (int64_t *)malloc(
      sizeof(int64_t) * (st->job->width * st->job->channels + 1));
  if (!vrow) {
    st->failed = 1;
    return NULL;
  }
  run_rows(st->job, st->y0, st->y1, vrow);
  free(vrow);
  return NULL;
}

/* Row-stripe parallelism, the same partitioning idea as
 * kleidicv_thread/src/kleidicv_thread.cpp:59-75: rows are independent because
 * every stripe recomputes its own vertical halo from src. */
static int run_job(const ko_job *j, int nthreads) {
  if (j->out_height == 0 || j->channels == 0) return KO_OK;
  if (nthreads < 1) nthreads = 1;
  if ((size_t)nthreads > j->out_height) nthreads = (int)j->out_height;
  ko_stripe st[256];
  pthread_t th[256];
  if (nthreads > 256) nthreads = 256;
  for (int i = 0; i < nthreads; ++i) {
    st[i].job = j;
    st[i].y0 = j->out_height * (size_t)i / (size_t)nthreads;
    st[i].y1 = j->out_height * (size_t)(i + 1) / (size_t)nthreads;
    st[i].failed = 0;
  }
  if (nthreads == 1) {
    stripe_main(&st[0]);
  } else {
    for (int i = 0; i < nthreads; ++i)
      pthread_create(&th[i], NULL, stripe_main, &st[i]);
    for (int i = 0; i < nthreads; ++i) pthread_join(th[i], NULL);
  }
  for (int i = 0; i < nthreads; ++i)
    if (st[i].failed) return KO_ALLOCATION;
  return KO_OK;
}

/* ------------------------------------------------------------------------ */
/* Validation helpers (utils.h:379-430). */
static int fixed_border_ok(int border) {
  return border == KO_BORDER_REPLICATE || border == KO_BORDER_REFLECT ||
         border == KO_BORDER_WRAP || border == KO_BORDER_REVERSE;
}

static int border_ok(int border, int ext) {
  return fixed_border_ok(border) || (ext && border == KO_BORDER_CONSTANT);
}

static int image_size_ok(size_t w, size_t h) {
  size_t n;
  if (__builtin_mul_overflow(w, h, &n)) return 0;
  return n <= KO_MAX_IMAGE_PIXELS;
}

static int stride_misaligned(size_t stride, size_t height, size_t elem) {
  return height > 1 && (stride % elem) != 0;
}

/* gaussian_blur_is_implemented (gaussian_blur.h:38-82). */
static int gaussian_is_implemented(size_t w, size_t h, size_t kw, size_t kh,
                                   float sx, float sy, size_t c, int border,
                                   int ext) {
  if (kw != kh) return 0;
  if (kw < 3 || kw > 255) return 0;
  if ((kw & 1) != 1) return 0;
  if (!(sx == sy)) return 0;
  if (w < kw - 1 || h < kw - 1) return 0;
  if (c > KO_MAX_CHANNELS) return 0;
  if (kw > 9 && kw != 15 && kw != 21) {
    if (border != KO_BORDER_REPLICATE && !(ext && border_ok(border, ext)))
      return 0;
    const size_t margin = kw / 2;
    const size_t aligned = (margin + 7) / 8 * 8;
    if (w < aligned + margin) return 0;
  }
  return 1;
}

static const int kBinomial3[] = {1, 2, 1};
static const int kBinomial5[] = {1, 4, 6, 4, 1};
static const int kBinomial7[] = {2, 7, 14, 18, 14, 7, 2};
static const int kBinomial9[] = {4, 13, 30, 51, 60, 51, 30, 13, 4};

int ko_gaussian_blur_u8(const uint8_t *src, size_t src_stride, uint8_t *dst,
                        size_t dst_stride, size_t width, size_t height,
                        size_t channels, size_t kernel_width,
                        size_t kernel_height, float sigma_x, float sigma_y,
                        int border_type, int ext, int border_value,
                        int nthreads) {
  /* gaussian_blur_api.cpp:28-37 then gaussian_blur.h:86-95 */
  if (!border_ok(border_type, ext)) return KO_NOT_IMPLEMENTED;
  if (!gaussian_is_implemented(width, height, kernel_width, kernel_height,
                               sigma_x, sigma_y, channels, border_type, ext))
    return KO_NOT_IMPLEMENTED;
  if (!src || !dst) return KO_NULL_POINTER;
  if (!image_size_ok(width, height)) return KO_RANGE;

  ko_job j;
  memset(&j, 0, sizeof(j));
  j.ksize = (int)kernel_width;
  j.border = border_type;
  j.border_value = border_value;
  j.width = width;
  j.height = height;
  j.channels = channels;
  j.out_width = width;
  j.out_height = height;
  j.src = src;
  j.src_stride = src_stride;
  j.dst = dst;
  j.dst_stride = dst_stride;
  j.elem_size = 1;

  const int fixed = kernel_width <= 9 || kernel_width == 15 ||
                    kernel_width == 21;
  if (fixed && kernel_width <= 9 && sigma_x == 0.0f) {
    const int *c = kernel_width == 3   ? kBinomial3
                   : kernel_width == 5 ? kBinomial5
                   : kernel_width == 7 ? kBinomial7
                                       : kBinomial9;
    j.mode = M_BINOM;
    j.shift = kernel_width == 3 ? 4 : kernel_width == 5 ? 8
              : kernel_width == 7                       ? 12
                                                        : 16;
    for (int t = 0; t < j.ksize; ++t) j.wy[t] = j.wx[t] = c[t];
    return run_job(&j, nthreads);
  }

  uint8_t half[128];
  const size_t half_size = kernel_width / 2 + 1;
  if (!ko_gaussian_half_kernel(half, half_size, sigma_x)) {
    /* gaussian_blur_fixed_neon.cpp:565-573: all weight in the middle tap. */
    for (size_t y = 0; y < height; ++y)
      memcpy(dst + y * dst_stride, src + y * src_stride, width * channels);
    return KO_OK;
  }
  j.mode = M_SIGMA;
  j.arbitrary = !fixed;
  j.vert_saturates = width * channels >= 16;
  j.arb_border_len = (channels * (kernel_width / 2) + 7) / 8 * 8;
  for (int t = 0; t < j.ksize; ++t) {
    const int hi = t < (int)half_size ? t : j.ksize - 1 - t;
    j.wy[t] = j.wx[t] = half[hi];
  }
  return run_job(&j, nthreads);
}

/* ------------------------------------------------------------------------ */
/* separable_filter_2d_api.cpp:12-31 then separable_filter_2d_neon.cpp:223-249 */
static int separable_common(const void *src, size_t src_stride, void *dst,
                            size_t dst_stride, size_t width, size_t height,
                            size_t channels, const void *kx, size_t kw,
                            const void *ky, size_t kh, int border, int ext,
                            size_t elem) {
  if (kw != 5 || kh != 5) return KO_NOT_IMPLEMENTED;
  if (width < kw - 1 || height < kw - 1) return KO_NOT_IMPLEMENTED;
  if (!border_ok(border, ext)) return KO_NOT_IMPLEMENTED;
  if (!src) return KO_NULL_POINTER;
  if (stride_misaligned(src_stride, height, elem)) return KO_ALIGNMENT;
  if (!dst) return KO_NULL_POINTER;
  if (stride_misaligned(dst_stride, height, elem)) return KO_ALIGNMENT;
  if (!image_size_ok(width, height)) return KO_RANGE;
  if (!kx || !ky) return KO_NULL_POINTER;
  if (channels > KO_MAX_CHANNELS) return KO_NOT_IMPLEMENTED;
  return KO_OK;
}

static int separable_run(int mode, const void *src, size_t src_stride,
                         void *dst, size_t dst_stride, size_t width,
                         size_t height, size_t channels, const int64_t *kx,
                         const int64_t *ky, int border, int border_value,
                         size_t elem, int nthreads) {
  ko_job j;
  memset(&j, 0, sizeof(j));
  j.mode = mode;
  j.ksize = 5;
  for (int t = 0; t < 5; ++t) {
    j.wx[t] = kx[t];
    j.wy[t] = ky[t];
  }
  j.border = border;
  j.border_value = border_value;
  j.width = width;
  j.height = height;
  j.channels = channels;
  j.out_width = width;
  j.out_height = height;
  j.src = (const uint8_t *)src;
  j.src_stride = src_stride;
  j.dst = (uint8_t *)dst;
  j.dst_stride = dst_stride;
  j.elem_size = elem;
  return run_job(&j, nthreads);
}

int ko_separable_filter_2d_u8(const uint8_t *src, size_t src_stride,
                              uint8_t *dst, size_t dst_stride, size_t width,
                              size_t height, size_t channels,
                              const uint8_t *kernel_x, size_t kernel_width,
                              const uint8_t *kernel_y, size_t kernel_height,
                              int border_type, int ext, int border_value,
                              int nthreads) {
  int e = separable_common(src, src_stride, dst, dst_stride, width, height,
                           channels, kernel_x, kernel_width, kernel_y,
                           kernel_height, border_type, ext, 1);
  if (e != KO_OK) return e;
  int64_t kx[5], ky[5];
  for (int t = 0; t < 5; ++t) {
    kx[t] = kernel_x[t];
    ky[t] = kernel_y[t];
  }
  return separable_run(M_SEP_U8, src, src_stride, dst, dst_stride, width,
                       height, channels, kx, ky, border_type,
                       border_value & 0xFF, 1, nthreads);
}

int ko_separable_filter_2d_u16(const uint16_t *src, size_t src_stride,
                               uint16_t *dst, size_t dst_stride, size_t width,
                               size_t height, size_t channels,
                               const uint16_t *kernel_x, size_t kernel_width,
                               const uint16_t *kernel_y, size_t kernel_height,
                               int border_type, int ext, int border_value,
                               int nthreads) {
  int e = separable_common(src, src_stride, dst, dst_stride, width, height,
                           channels, kernel_x, kernel_width, kernel_y,
                           kernel_height, border_type, ext, 2);
  if (e != KO_OK) return e;
  int64_t kx[5], ky[5];
  for (int t = 0; t < 5; ++t) {
    kx[t] = kernel_x[t];
    ky[t] = kernel_y[t];
  }
  return separable_run(M_SEP_U16, src, src_stride, dst, dst_stride, width,
                       height, channels, kx, ky, border_type,
                       border_value & 0xFFFF, 2, nthreads);
}

int ko_separable_filter_2d_s16(const int16_t *src, size_t src_stride,
                               int16_t *dst, size_t dst_stride, size_t width,
                               size_t height, size_t channels,
                               const int16_t *kernel_x, size_t kernel_width,
                               const int16_t *kernel_y, size_t kernel_height,
                               int border_type, int border_value,
                               int nthreads) {
  int e = separable_common(src, src_stride, dst, dst_stride, width, height,
                           channels, kernel_x, kernel_width, kernel_y,
                           kernel_height, border_type, 1, 2);
  if (e != KO_OK) return e;
  int64_t kx[5], ky[5];
  for (int t = 0; t < 5; ++t) {
    kx[t] = kernel_x[t];
    ky[t] = kernel_y[t];
  }
  return separable_run(M_SEP_S16, src, src_stride, dst, dst_stride, width,
                       height, channels, kx, ky, border_type,
                       (int16_t)border_value, 2, nthreads);
}

/* ------------------------------------------------------------------------ */
/* blur_and_downsample_api.cpp:17-34 then blur_and_downsample_neon.cpp:322-336
 */
int ko_blur_and_downsample_u8(const uint8_t *src, size_t src_stride,
                              size_t src_width, size_t src_height,
                              uint8_t *dst, size_t dst_stride, size_t channels,
                              int border_type, int ext, int border_value,
                              int nthreads) {
  if (!(src_width >= 4 && src_height >= 4 && channels >= 1 &&
        channels <= KO_MAX_CHANNELS))
    return KO_NOT_IMPLEMENTED;
  if (!border_ok(border_type, ext)) return KO_NOT_IMPLEMENTED;
  if (!src || !dst) return KO_NULL_POINTER;
  if (!image_size_ok(src_width, src_height)) return KO_RANGE;

  ko_job j;
  memset(&j, 0, sizeof(j));
  j.mode = M_BLURDOWN;
  j.ksize = 5;
  for (int t = 0; t < 5; ++t) j.wy[t] = j.wx[t] = kBinomial5[t];
  j.border = border_type;
  j.border_value = border_value & 0xFF;
  j.width = src_width;
  j.height = src_height;
  j.channels = channels;
  j.out_width = (src_width + 1) / 2;
  j.out_height = (src_height + 1) / 2;
  j.src = src;
  j.src_stride = src_stride;
  j.dst = dst;
  j.dst_stride = dst_stride;
  j.elem_size = 1;
  return run_job(&j, nthreads);
}

/* ------------------------------------------------------------------------ */
/* sobel_api.cpp:22-31 (sobel_is_implemented, filters/sobel.h:30-33), then
 * sobel_neon.cpp:131-162 / :165-196: src and dst pointer/stride checks (a u8
 * stride cannot be misaligned), image size, channels, then a separable 3x3
 * pass with the REPLICATE border. */
static int sobel_run(int mode, const uint8_t *src, size_t src_stride,
                     int16_t *dst, size_t dst_stride, size_t width,
                     size_t height, size_t channels, int nthreads) {
  if (!(width >= 2 && height >= 2)) return KO_NOT_IMPLEMENTED;
  if (!src) return KO_NULL_POINTER;
  if (!dst) return KO_NULL_POINTER;
  if (stride_misaligned(dst_stride, height, 2)) return KO_ALIGNMENT;
  if (!image_size_ok(width, height)) return KO_RANGE;
  if (channels > KO_MAX_CHANNELS) return KO_NOT_IMPLEMENTED;

  static const int64_t smooth[3] = {1, 2, 1}, diff[3] = {-1, 0, 1};
  ko_job j;
  memset(&j, 0, sizeof(j));
  j.mode = mode;
  j.ksize = 3;
  for (int t = 0; t < 3; ++t) {
    j.wy[t] = mode == M_SOBEL_X ? smooth[t] : diff[t];
    j.wx[t] = mode == M_SOBEL_X ? diff[t] : smooth[t];
  }
  j.border = KO_BORDER_REPLICATE;
  j.width = width;
  j.height = height;
  j.channels = channels;
  j.out_width = width;
  j.out_height = height;
  j.src = src;
  j.src_stride = src_stride;
  j.dst = (uint8_t *)dst;
  j.dst_stride = dst_stride;
  j.elem_size = 1;
  return run_job(&j, nthreads);
}

int ko_sobel_3x3_horizontal_s16_u8(const uint8_t *src, size_t src_stride,
                                   int16_t *dst, size_t dst_stride,
                                   size_t width, size_t height,
                                   size_t channels, int nthreads) {
  return sobel_run(M_SOBEL_X, src, src_stride, dst, dst_stride, width, height,
                   channels, nthreads);
}

int ko_sobel_3x3_vertical_s16_u8(const uint8_t *src, size_t src_stride,
                                 int16_t *dst, size_t dst_stride, size_t width,
                                 size_t height, size_t channels,
                                 int nthreads) {
  return sobel_run(M_SOBEL_Y, src, src_stride, dst, dst_stride, width, height,
                   channels, nthreads);
}

/* ------------------------------------------------------------------------ */
/* Fills out[i * ksize + t] = map(i + t - ksize/2) for i in [0, n): the
 * absolute source index each tap of each position reads, i.e. the quantity
 * the reference's FixedBorderInfo<K>::offsets_with_border(i) encodes
 * relative to i.  Used to pin ko_border_map against those tables. */
void ko_border_table(int ksize, long n, int border, long *out) {
  const long r = ksize / 2;
  for (long i = 0; i < n; ++i)
    for (long t = 0; t < ksize; ++t)
      out[i * ksize + t] = ko_border_map(i + t - r, n, border);
}
