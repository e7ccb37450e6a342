// Generic two-pass Gaussian for arbitrary odd kernel sizes (11..255, the
// reference's kleidicv/src/filters/gaussian_blur_arbitrary_neon.cpp) and for
// any generated kernel whose weights do not sum to 256.
//
// Pass 1 writes the u8 vertical intermediate of the whole image into a
// scratch image; pass 2 stages each row segment (plus its border-mapped halo)
// in shared memory and applies the horizontal taps.  Arithmetic is per
// element in 32 bits and reproduces, element by element, which rounding the
// reference applied: the arbitrary-size vector paths add the rounding
// constant with saturation (vqaddq_u16, :193-194, :306-307), its border
// vector paths narrow with vrshrn (:340, :374) and its scalar paths cast a
// u32 sum to u8 (:232-244, :381-383); these differ only when a sum of weights
// above 256 lets a 16-bit accumulator pass 65535.
#include <cuda_runtime.h>
#include <stdint.h>

#include "launch.h"
#include "sepfused.cuh"

namespace kcv {

namespace {

__device__ __forceinline__ uint32_t round_wrap(uint32_t acc) { return ((acc + 128u) >> 8) & 0xFFu; }
__device__ __forceinline__ uint32_t round_sat(uint32_t acc) {
  const uint32_t a = acc + 128u;
  return (a > 0xFFFFu ? 0xFFFFu : a) >> 8;
}

__device__ __forceinline__ uint32_t weight(const GenericJob &j, int t) {
  const int r = j.ksize / 2;
  return j.half[t <= r ? t : j.ksize - 1 - t];
}

// Destination rows per thread in pass 1: few enough that a 4K image fills
// the GPU more than once (16 rows gave 0.44 waves on 3840x2160x1).
constexpr int kRowsPerThread = 4;
constexpr int kHThreads = 256;
constexpr int kHElems = 4 * kHThreads;  // row elements per CTA in pass 2

// The full kernel's weights (ksize <= 255) into shared memory, once per CTA:
// the tap loops then read them without the mirror select.
__device__ __forceinline__ void stage_weights(const GenericJob &j, uint32_t *wts) {
  for (int t = threadIdx.x; t < j.ksize; t += blockDim.x) wts[t] = weight(j, t);
  __syncthreads();
}

__global__ void __launch_bounds__(256) generic_vertical(const __grid_constant__ GenericJob j,
                                                        uint8_t *vbuf, size_t vstride) {
  __shared__ uint32_t wts[256];
  stage_weights(j, wts);
  const long wc = static_cast<long>(j.width) * j.channels;
  const long x = (static_cast<long>(blockIdx.x) * blockDim.x + threadIdx.x) * 4;
  if (x >= wc) return;
  const int ne = static_cast<int>(wc - x < 4 ? wc - x : 4);
  const int r = j.ksize / 2;
  // Whole 4-byte words when the column's words are 4-byte aligned in every
  // row.
  const bool words = ne == 4 && ((reinterpret_cast<uintptr_t>(j.src + x) | static_cast<uintptr_t>(j.src_stride)) & 3) == 0;
  // Row blocks loop over the grid's y extent, which the hardware caps at 65535.
  for (long yb = blockIdx.y; yb * kRowsPerThread < j.height; yb += gridDim.y) {
    const int y0 = static_cast<int>(yb * kRowsPerThread);
    const int y1 = min(y0 + kRowsPerThread, j.height);
    if (words && y0 >= r && y1 - 1 + r < j.height) {
      // Every tap row inside the image: step a row pointer, no border map.
      for (int y = y0; y < y1; ++y) {
        uint32_t acc[4] = {0, 0, 0, 0};
        const uint8_t *row = j.src + static_cast<int64_t>(y - r) * j.src_stride + x;
        for (int t = 0; t < j.ksize; ++t, row += j.src_stride) {
          const uint32_t g = wts[t];
          const uint32_t w = __ldg(reinterpret_cast<const uint32_t *>(row));
          acc[0] += g * (w & 0xFFu);
          acc[1] += g * ((w >> 8) & 0xFFu);
          acc[2] += g * ((w >> 16) & 0xFFu);
          acc[3] += g * (w >> 24);
        }
        uint32_t o = 0;
#pragma unroll
        for (int e = 0; e < 4; ++e)
          o |= (j.vert_saturates ? round_sat(acc[e]) : round_wrap(acc[e])) << (8 * e);
        uint8_t *out = vbuf + static_cast<int64_t>(y) * vstride + x;
        if ((reinterpret_cast<uintptr_t>(out) & 3) == 0) {
          *reinterpret_cast<uint32_t *>(out) = o;
        } else {
          for (int e = 0; e < 4; ++e) out[e] = static_cast<uint8_t>(o >> (8 * e));
        }
      }
      continue;
    }
    for (int y = y0; y < y1; ++y) {
      uint32_t acc[4] = {0, 0, 0, 0};
      for (int t = 0; t < j.ksize; ++t) {
        const int ry = map_index(y + t - r, j.height, j.border);
        const uint32_t g = wts[t];
        if (ry < 0) {
          const uint32_t bv = static_cast<uint32_t>(j.border_value) & 0xFFu;
          for (int e = 0; e < 4; ++e) acc[e] += g * bv;
        } else {
          const uint8_t *row = j.src + static_cast<int64_t>(ry) * j.src_stride + x;
          if (ne == 4 && (reinterpret_cast<uintptr_t>(row) & 3) == 0) {
            const uint32_t w = __ldg(reinterpret_cast<const uint32_t *>(row));
            acc[0] += g * (w & 0xFFu);
            acc[1] += g * ((w >> 8) & 0xFFu);
            acc[2] += g * ((w >> 16) & 0xFFu);
            acc[3] += g * (w >> 24);
          } else {
            for (int e = 0; e < ne; ++e) acc[e] += g * __ldg(row + e);
          }
        }
      }
      uint8_t *out = vbuf + static_cast<int64_t>(y) * vstride + x;
      for (int e = 0; e < ne; ++e)
        out[e] = static_cast<uint8_t>(j.vert_saturates ? round_sat(acc[e]) : round_wrap(acc[e]));
    }
  }
}

__device__ __forceinline__ bool h_saturates(const GenericJob &j, long x, long wc) {
  if (!j.arbitrary) return false;
  const long bl = j.arb_border_len;
  if (wc <= 2 * bl || x < bl || x >= wc - bl) return false;
  return wc - 2 * bl >= 16;
}

// Right-border lane channel of the arbitrary-size path.  The reference
// computes the last arb_border_len elements of a row with 8-lane vectors that
// start at width*channels - arb_border_len; for the right-hand tap at distance
// d columns, a vector starting at xv whose lanes xv + c*d .. +7 all lie past
// the row end takes its replicated lanes from an index pattern that gives
// lanes 8-q..7 channel lane+c-8 of the last pixel, q = (xv + c*d) % c, instead
// of channel (q + lane) % c (border_generic_neon.h:80-98,
// gaussian_blur_arbitrary_neon.cpp:346-377).  Returns that channel, or -1
// where the lane is exact.
__device__ __forceinline__ int right_lane_channel(long e, int d, int c, long wc, long bl) {
  const long xv = wc - bl + (e - (wc - bl)) / 8 * 8;
  const int lane = static_cast<int>(e - xv);
  const long start = xv + static_cast<long>(c) * d;
  if (start < wc) return -1;
  const int q = static_cast<int>((start - wc) % c);
  if (q == 0 || lane < 8 - q) return -1;
  return lane + c - 8;
}

__global__ void __launch_bounds__(kHThreads) generic_horizontal(const __grid_constant__ GenericJob j,
                                                                const uint8_t *vbuf,
                                                                size_t vstride) {
  // seg holds row elements [x0 - halo, x0 + kHElems + halo) of the
  // intermediate, element x0 at the 4-aligned byte `lead`.
  extern __shared__ __align__(16) uint8_t seg_mem[];
  __shared__ uint32_t wts[256];
  stage_weights(j, wts);
  const int c = j.channels;
  const int r = j.ksize / 2;
  const long wc = static_cast<long>(j.width) * c;
  const long x0 = static_cast<long>(blockIdx.x) * kHElems;
  const int halo = r * c;
  const int lead = (halo + 3) & ~3;
  uint8_t *seg = seg_mem + (lead - halo);  // seg[i]: element x0 - halo + i
  const uint32_t *seg32 = reinterpret_cast<const uint32_t *>(seg_mem);
  const int n = static_cast<int>(wc - x0 < kHElems ? wc - x0 : kHElems);  // interior elements
  const bool words = ((reinterpret_cast<uintptr_t>(vbuf) | static_cast<uintptr_t>(vstride)) & 3) == 0;
  const bool right_quirk = j.arbitrary && c > 1 && x0 + kHElems > wc - j.arb_border_len;
  const int local0 = threadIdx.x * 4;  // the thread's first element of the segment
  const int ne = static_cast<int>(n - local0 < 4 ? n - local0 : 4);
  // Rows loop over the grid's y extent, which the hardware caps at 65535.
  for (int y = blockIdx.y; y < j.height; y += gridDim.y) {
    const uint8_t *vrow = vbuf + static_cast<int64_t>(y) * vstride;
    __syncthreads();  // the previous row's reads of seg are done
    // The interior as words where the rows allow, the rest byte by byte.
    const int nw = words ? n / 4 : 0;
    for (int q = threadIdx.x; q < nw; q += blockDim.x)
      reinterpret_cast<uint32_t *>(seg_mem + lead)[q] = reinterpret_cast<const uint32_t *>(vrow + x0)[q];
    for (int i = 4 * nw + threadIdx.x; i < n; i += blockDim.x) seg[halo + i] = vrow[x0 + i];
    // The halos, with the border resolved per element.
    for (int i = threadIdx.x; i < 2 * halo; i += blockDim.x) {
      const int idx = i < halo ? i : n + i;  // [0, halo) and [halo + n, 2 halo + n)
      const long xe = x0 - halo + idx;
      uint8_t v;
      if (xe >= 0 && xe < wc) {
        v = vrow[xe];
      } else {
        const long col = xe >= 0 ? xe / c : -((-xe + c - 1) / c);
        const int ch = static_cast<int>(xe - col * c);
        const int mc = map_index(static_cast<int>(col), j.width, j.border);
        v = mc < 0 ? static_cast<uint8_t>(j.v_const) : vrow[static_cast<long>(mc) * c + ch];
      }
      seg[idx] = v;
    }
    __syncthreads();
    if (ne <= 0) continue;
    // Tap t of the thread's 4 elements: the 4 bytes at segment position
    // local0 + t c, from the two words around them.
    uint32_t acc[4] = {0, 0, 0, 0};
    int p = (lead - halo) + local0;  // byte of tap 0, element 0
    for (int t = 0; t < j.ksize; ++t, p += c) {
      const uint32_t g = wts[t];
      const uint32_t v = __funnelshift_r(seg32[p >> 2], seg32[(p >> 2) + 1], 8 * (p & 3));
      acc[0] += g * (v & 0xFFu);
      acc[1] += g * ((v >> 8) & 0xFFu);
      acc[2] += g * ((v >> 16) & 0xFFu);
      acc[3] += g * (v >> 24);
    }
    uint8_t *drow = j.dst + static_cast<int64_t>(y) * j.dst_stride;
    for (int k = 0; k < ne; ++k) {
      const int local = local0 + k;
      const long x = x0 + local;
      uint32_t a = acc[k];
      if (right_quirk && x >= wc - j.arb_border_len) {
        const uint8_t *last = vrow + wc - c;
        for (int d = 1; d <= r; ++d) {
          const int qc = right_lane_channel(x, d, c, wc, j.arb_border_len);
          if (qc >= 0) a = a - wts[r + d] * seg[local + (r + d) * c] + wts[r + d] * last[qc];
        }
      }
      drow[x] = static_cast<uint8_t>(h_saturates(j, x, wc) ? round_sat(a) : round_wrap(a));
    }
  }
}

}  // namespace

cudaError_t launch_generic_gaussian(const GenericJob &job, uint8_t *scratch, size_t scratch_stride,
                                    cudaStream_t stream) {
  const long wc = static_cast<long>(job.width) * job.channels;
  const long words = (wc + 3) / 4;
  const long row_blocks = (job.height + kRowsPerThread - 1) / kRowsPerThread;
  dim3 g1(static_cast<unsigned>((words + 255) / 256), static_cast<unsigned>(row_blocks < 65535 ? row_blocks : 65535));
  generic_vertical<<<g1, 256, 0, stream>>>(job, scratch, scratch_stride);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  // The segment (halos on either side, the interior from a 4-aligned byte)
  // and 8 bytes that the last taps' word reads may touch.
  const size_t halo = static_cast<size_t>(job.ksize / 2) * job.channels;
  const size_t smem = ((halo + 3) & ~static_cast<size_t>(3)) + kHElems + halo + 8;
  dim3 g2(static_cast<unsigned>((wc + kHElems - 1) / kHElems),
          static_cast<unsigned>(job.height < 65535 ? job.height : 65535));
  generic_horizontal<<<g2, kHThreads, smem, stream>>>(job, scratch, scratch_stride);
  return cudaGetLastError();
}

cudaError_t preload_generic_gaussian() {
  cudaFuncAttributes a;
  cudaError_t e = cudaFuncGetAttributes(&a, generic_vertical);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, generic_horizontal);
  return e;
}

}  // namespace kcv
