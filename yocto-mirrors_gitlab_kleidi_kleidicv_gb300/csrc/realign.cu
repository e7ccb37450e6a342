// Copies an image whose rows TMA cannot address (base or stride not a
// multiple of 16 bytes) into a scratch image with 16-byte aligned rows, so
// that the tiled stencil streams it through its TMA ring instead of loading
// every chunk synchronously.  One thread per 16-byte destination chunk: the
// two aligned 16-byte blocks around the source chunk when both lie inside the
// row (a funnel shift puts the bytes in place), the ragged row ends byte by
// byte (16 independent loads).  Adjacent threads share source blocks through
// L1, so DRAM sees the image about once.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "launch.h"
#include "sepfused.cuh"

namespace kcv {

namespace {

__global__ void __launch_bounds__(256) realign_rows(const uint8_t *src, int64_t src_stride, uint8_t *dst,
                                                    int64_t dst_stride, long row_bytes, int height) {
  const long chunks = (row_bytes + 15) / 16;
  const long total = chunks * height;
  for (long i = static_cast<long>(blockIdx.x) * blockDim.x + threadIdx.x; i < total;
       i += static_cast<long>(gridDim.x) * blockDim.x) {
    const long y = i / chunks;
    const long xb = 16 * (i - y * chunks);
    const uint8_t *row = src + y * src_stride;
    uint8_t *out = dst + y * dst_stride + xb;
    uint4 v;
    if (xb + 16 <= row_bytes && load_chunk_fast(row, xb, row_bytes, v)) {
      *reinterpret_cast<uint4 *>(out) = v;
    } else {
      // The ragged ends: all 16 byte loads in flight at once (a loop with a
      // runtime bound would wait for each before the next).
      const int n = static_cast<int>(row_bytes - xb < 16 ? row_bytes - xb : 16);
      uint8_t b[16];
#pragma unroll
      for (int k = 0; k < 16; ++k) b[k] = k < n ? __ldg(row + xb + k) : 0;
#pragma unroll
      for (int k = 0; k < 16; ++k)
        if (k < n) out[k] = b[k];
    }
  }
}

}  // namespace

cudaError_t launch_realign(const uint8_t *src, int64_t src_stride, uint8_t *dst, int64_t dst_stride,
                           long row_bytes, int height, int sm_count, cudaStream_t stream) {
  const long total = (row_bytes + 15) / 16 * height;
  // Grid-stride over the chunks: at most 8 CTAs of 256 threads per SM.
  const long blocks = std::max(1L, std::min((total + 255) / 256, 8L * std::max(sm_count, 1)));
  realign_rows<<<static_cast<unsigned>(blocks), 256, 0, stream>>>(src, src_stride, dst, dst_stride, row_bytes,
                                                                  height);
  return cudaGetLastError();
}

}  // namespace kcv
