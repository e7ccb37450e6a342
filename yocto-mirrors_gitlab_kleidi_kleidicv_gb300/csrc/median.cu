// Median blur on the GPU: kleidicv_median_blur_{s8,u8,u16,s16,u32,s32,f32}
// (kleidicv/src/filters/median_blur_api.cpp, validation in
// kleidicv/include/kleidicv/filters/median_blur.h:148-193).  The result is the
// median of the border-mapped K x K window of every element, which is unique,
// so any exact selection reproduces the reference's sorting networks
// (K = 3, 5, 7) and histograms (u8, K = 9..255).
//
//  * K <= 7: one thread per destination element and a block of rows.  The
//    window is read through the read-only cache as order-preserving unsigned
//    keys, and the median is selected by forgetful selection: keep the first
//    N/2 + 2 values, repeatedly move the smallest and largest to the ends by
//    compare-exchange passes, drop both (neither can be the median: equal
//    numbers are dropped below and above it) and take in the next value;
//    the last three hold the median.
//  * u8, K >= 9: Huang's sliding histogram.  A thread owns a run of
//    max(16, K/2) pixels of one row and channel and a 256-bin histogram in
//    shared memory (bins outermost, so the 64 threads of a block hit distinct
//    banks); moving one pixel right removes a column, adds a column and moves
//    the median bin by the count of values that crossed it.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "../../include/kleidicv_gpu.h"
#include "host.h"
#include "launch.h"
#include "sepfused.cuh"

namespace kcv {
namespace {

// Order-preserving unsigned keys.  Floats: sign-magnitude to offset binary
// (-0.0 orders just below +0.0).
template <typename T>
struct Key;
template <>
struct Key<uint8_t> {
  __device__ static uint32_t to(uint8_t v) { return v; }
  __device__ static uint8_t from(uint32_t k) { return static_cast<uint8_t>(k); }
};
template <>
struct Key<int8_t> {
  __device__ static uint32_t to(int8_t v) { return static_cast<uint8_t>(v) ^ 0x80u; }
  __device__ static int8_t from(uint32_t k) { return static_cast<int8_t>(k ^ 0x80u); }
};
template <>
struct Key<uint16_t> {
  __device__ static uint32_t to(uint16_t v) { return v; }
  __device__ static uint16_t from(uint32_t k) { return static_cast<uint16_t>(k); }
};
template <>
struct Key<int16_t> {
  __device__ static uint32_t to(int16_t v) { return static_cast<uint16_t>(v) ^ 0x8000u; }
  __device__ static int16_t from(uint32_t k) { return static_cast<int16_t>(k ^ 0x8000u); }
};
template <>
struct Key<uint32_t> {
  __device__ static uint32_t to(uint32_t v) { return v; }
  __device__ static uint32_t from(uint32_t k) { return k; }
};
template <>
struct Key<int32_t> {
  __device__ static uint32_t to(int32_t v) { return static_cast<uint32_t>(v) ^ 0x80000000u; }
  __device__ static int32_t from(uint32_t k) { return static_cast<int32_t>(k ^ 0x80000000u); }
};
template <>
struct Key<float> {
  __device__ static uint32_t to(float v) {
    const uint32_t b = __float_as_uint(v);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
  }
  __device__ static float from(uint32_t k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k);
  }
};

__device__ __forceinline__ void cex(uint32_t &lo, uint32_t &hi) {
  const uint32_t a = min(lo, hi), b = max(lo, hi);
  lo = a;
  hi = b;
}

// Forgetful selection over a[0..N) (N odd); returns the median key.  Step S
// works on the buffer a[S .. R) (R = N/2 + 2) and takes in a[R + S].
template <int N, int S = 0>
__device__ __forceinline__ uint32_t forgetful(uint32_t (&a)[N]) {
  constexpr int R = N / 2 + 2;
  if constexpr (R + S == N) {
    // Three values remain: a[S], a[S+1], a[S+2].
    uint32_t x = a[S], y = a[S + 1], z = a[S + 2];
    cex(x, y);
    cex(y, z);
    cex(x, y);
    return y;
  } else {
    static_for<S + 1, R>([&](auto ic) { cex(a[S], a[decltype(ic)::value]); });       // min -> a[S]
    static_for<S + 1, R - 1>([&](auto ic) { cex(a[decltype(ic)::value], a[R - 1]); });  // max -> a[R-1]
    a[R - 1] = a[R + S];  // drop both ends, take in the next value
    return forgetful<N, S + 1>(a);
  }
}

template <typename T, int K>
__global__ void __launch_bounds__(128) median_small_kernel(const uint8_t *src, int64_t src_stride,
                                                           uint8_t *dst, int64_t dst_stride, int w,
                                                           int h, int c, int border,
                                                           int rows_per_block) {
  constexpr int R = K / 2;
  const int xe = blockIdx.x * blockDim.x + threadIdx.x;  // element index in the row
  if (xe >= w * c) return;
  const int col = xe / c, ch = xe - col * c;
  int cidx[K];
#pragma unroll
  for (int d = 0; d < K; ++d) cidx[d] = map_index(col + d - R, w, border) * c + ch;
  // Row blocks loop over the grid's y extent, which the hardware caps at 65535.
  for (long yb = blockIdx.y; yb * rows_per_block < h; yb += gridDim.y) {
    const int y0 = static_cast<int>(yb * rows_per_block), y1 = min(h, y0 + rows_per_block);
    for (int y = y0; y < y1; ++y) {
      uint32_t a[K * K];
#pragma unroll
      for (int dy = 0; dy < K; ++dy) {
        const T *row = reinterpret_cast<const T *>(
            src + static_cast<int64_t>(map_index(y + dy - R, h, border)) * src_stride);
#pragma unroll
        for (int dx = 0; dx < K; ++dx) a[dy * K + dx] = Key<T>::to(__ldg(row + cidx[dx]));
      }
      reinterpret_cast<T *>(dst + static_cast<int64_t>(y) * dst_stride)[xe] =
          Key<T>::from(forgetful<K * K>(a));
    }
  }
}

constexpr int kHistThreads = 64;

// Pixels per thread: at least K/2, so that the O(K^2) start costs no more per
// pixel than the O(K) steps, and otherwise short, so that a 1080p image still
// gives tens of thousands of threads.
int hist_run(int k) { return std::max(16, (k / 2 + 15) / 16 * 16); }

__global__ void __launch_bounds__(kHistThreads) median_hist_kernel(const uint8_t *src,
                                                                  int64_t src_stride,
                                                                  uint8_t *dst,
                                                                  int64_t dst_stride, int w,
                                                                  int h, int c, int k,
                                                                  int border, int run) {
  __shared__ uint16_t hist[256 * kHistThreads];  // [bin][thread]; counts <= 255 * 255
  const int tid = threadIdx.x;
  const int g = blockIdx.x * kHistThreads + tid;  // (segment, channel) item of a row
  const int ch = g % c, seg = g / c;
  const int x0 = seg * run;
  if (x0 >= w) return;  // no __syncthreads below: threads are independent
  const int x1 = min(w, x0 + run);
  const int r = k / 2;
  const int m = (k * k - 1) / 2;  // rank of the median
  auto value = [&](int yy, int xx) -> int {
    const uint8_t *row = src + static_cast<int64_t>(map_index(yy, h, border)) * src_stride;
    return __ldg(row + map_index(xx, w, border) * c + ch);
  };
  // Rows loop over the grid's y extent, which the hardware caps at 65535.
  for (int y = blockIdx.y; y < h; y += gridDim.y) {
    for (int b = 0; b < 256; ++b) hist[b * kHistThreads + tid] = 0;
    for (int dy = -r; dy <= r; ++dy)
      for (int dx = -r; dx <= r; ++dx) ++hist[value(y + dy, x0 + dx) * kHistThreads + tid];
    int med = 0, lt = 0;
    while (lt + hist[med * kHistThreads + tid] <= m) lt += hist[(med++) * kHistThreads + tid];
    uint8_t *drow = dst + static_cast<int64_t>(y) * dst_stride;
    drow[x0 * c + ch] = static_cast<uint8_t>(med);
    for (int x = x0 + 1; x < x1; ++x) {
      for (int dy = -r; dy <= r; ++dy) {
        const int out = value(y + dy, x - 1 - r), in = value(y + dy, x + r);
        --hist[out * kHistThreads + tid];
        ++hist[in * kHistThreads + tid];
        lt += (in < med) - (out < med);
      }
      while (lt > m) lt -= hist[(--med) * kHistThreads + tid];
      while (lt + hist[med * kHistThreads + tid] <= m) lt += hist[(med++) * kHistThreads + tid];
      drow[x * c + ch] = static_cast<uint8_t>(med);
    }
  }
}

template <typename T, int K>
cudaError_t launch_small(const MedianJob &j, cudaStream_t s) {
  const int rows_per_block = 4;
  const int row_blocks = (j.height + rows_per_block - 1) / rows_per_block;
  dim3 grid(static_cast<unsigned>((j.width * j.channels + 127) / 128),
            static_cast<unsigned>(row_blocks < 65535 ? row_blocks : 65535));
  median_small_kernel<T, K><<<grid, 128, 0, s>>>(j.src, j.src_stride, j.dst, j.dst_stride,
                                                  j.width, j.height, j.channels, j.border,
                                                  rows_per_block);
  return cudaGetLastError();
}

template <typename T>
cudaError_t launch_typed(const MedianJob &j, cudaStream_t s) {
  switch (j.ksize) {
    case 3: return launch_small<T, 3>(j, s);
    case 5: return launch_small<T, 5>(j, s);
    case 7: return launch_small<T, 7>(j, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace

cudaError_t launch_median(const MedianJob &j, cudaStream_t s) {
  if (j.ksize > 7) {
    if (j.elem != MEDIAN_U8) return cudaErrorInvalidValue;
    const int run = hist_run(j.ksize);
    const int items = j.channels * ((j.width + run - 1) / run);
    dim3 grid(static_cast<unsigned>((items + kHistThreads - 1) / kHistThreads),
              static_cast<unsigned>(j.height < 65535 ? j.height : 65535));
    median_hist_kernel<<<grid, kHistThreads, 0, s>>>(j.src, j.src_stride, j.dst, j.dst_stride,
                                                     j.width, j.height, j.channels, j.ksize,
                                                     j.border, run);
    return cudaGetLastError();
  }
  switch (j.elem) {
    case MEDIAN_S8: return launch_typed<int8_t>(j, s);
    case MEDIAN_U8: return launch_typed<uint8_t>(j, s);
    case MEDIAN_U16: return launch_typed<uint16_t>(j, s);
    case MEDIAN_S16: return launch_typed<int16_t>(j, s);
    case MEDIAN_U32: return launch_typed<uint32_t>(j, s);
    case MEDIAN_S32: return launch_typed<int32_t>(j, s);
    case MEDIAN_F32: return launch_typed<float>(j, s);
  }
  return cudaErrorInvalidValue;
}

}  // namespace kcv
