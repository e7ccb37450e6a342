// kleidicv_gpu_gaussian_blur_u8_noalloc: the arbitrary-size Gaussian with its
// intermediate image in a fixed device buffer instead of the context's pool.
//
// The buffer is a file-scope __device__ array, part of the library's device
// image.  Its address is resolved once per device (cudaGetSymbolAddress with
// that device current) and cached; every call after that only validates and
// enqueues: no cudaMalloc / cudaFree / pool routine, no context.
#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <mutex>

#include "../../include/kleidicv_gpu.h"
#include "host.h"
#include "launch.h"

namespace kcv {
namespace {

// The intermediate (vertical-pass) image: rows of ceil16(width*channels)
// bytes.  No initial contents are needed: generic_vertical writes every byte
// that generic_horizontal reads.
__device__ __align__(256) uint8_t g_noalloc_scratch[KLEIDICV_GPU_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
uint8_t *g_scratch_addr[kMaxDevices];  // nullptr until the device's set-up ran

// One-time set-up for the current device: checks it runs sm_103 code, loads
// the two kernels and resolves the buffer's device address.
kleidicv_error_t scratch_for_current_device(uint8_t **out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return KLEIDICV_GPU_ERROR_NO_DEVICE;
  }
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_addr[dev]) {
    int major = 0, minor = 0;
    if (cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev) != cudaSuccess ||
        major != 10 || minor != 3) {
      cudaGetLastError();
      return KLEIDICV_GPU_ERROR_NO_DEVICE;
    }
    if (preload_generic_gaussian() != cudaSuccess) {
      cudaGetLastError();
      return KLEIDICV_GPU_ERROR_CUDA;
    }
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || p == nullptr) {
      cudaGetLastError();
      return KLEIDICV_GPU_ERROR_CUDA;
    }
    g_scratch_addr[dev] = static_cast<uint8_t *>(p);
  }
  *out = g_scratch_addr[dev];
  return KLEIDICV_OK;
}

}  // namespace
}  // namespace kcv

using namespace kcv;

extern "C" kleidicv_error_t kleidicv_gpu_gaussian_blur_u8_noalloc(
    const uint8_t *src, size_t src_stride, uint8_t *dst, size_t dst_stride, size_t width,
    size_t height, size_t channels, size_t kernel_width, size_t kernel_height, float sigma_x,
    float sigma_y, kleidicv_border_type_t border_type, void *stream) {
  Prepared p;
  kleidicv_error_t e =
      prepare_gaussian(src, src_stride, dst, dst_stride, width, height, channels, kernel_width,
                       kernel_height, sigma_x, sigma_y, static_cast<int>(border_type),
                       /*ext=*/false, /*border_value=*/0, &p);
  if (e != KLEIDICV_OK) return e;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  switch (p.kind) {
    case Prepared::NOTHING:
      return KLEIDICV_OK;
    case Prepared::FUSED:
      return KLEIDICV_ERROR_NOT_IMPLEMENTED;
    case Prepared::COPY:
      if (cudaMemcpy2DAsync(p.dst, p.dst_stride, p.src, p.src_stride, p.row_bytes, p.rows,
                            cudaMemcpyDeviceToDevice, s) != cudaSuccess) {
        cudaGetLastError();
        return KLEIDICV_GPU_ERROR_CUDA;
      }
      return KLEIDICV_OK;
    case Prepared::GENERIC: {
      const GenericJob &g = p.generic;
      const size_t vstride = (static_cast<size_t>(g.width) * g.channels + 15) / 16 * 16;
      if (vstride * static_cast<size_t>(g.height) > KLEIDICV_GPU_NOALLOC_SCRATCH_BYTES)
        return KLEIDICV_ERROR_RANGE;
      uint8_t *scratch = nullptr;
      e = scratch_for_current_device(&scratch);
      if (e != KLEIDICV_OK) return e;
      if (launch_generic_gaussian(g, scratch, vstride, s) != cudaSuccess) {
        cudaGetLastError();
        return KLEIDICV_GPU_ERROR_CUDA;
      }
      return KLEIDICV_OK;
    }
  }
  return KLEIDICV_OK;
}
