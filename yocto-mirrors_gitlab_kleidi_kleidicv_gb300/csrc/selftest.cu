// Failure-path self-test of the bounded device-side waits: a kernel waits on
// an mbarrier that nothing ever arrives at, gives up after the requested
// limit and reports through the context's error flag, exactly like a fused
// kernel whose copies never land.  The context stays usable afterwards.
#include <cuda_runtime.h>

#include "../../include/kleidicv_gpu.h"
#include "host.h"
#include "ptx.cuh"

namespace kcv {
namespace {

__global__ void bounded_wait_selftest(int *err_flag, uint64_t limit_ns) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
    if (!mbar_wait_bounded(&bar, 0u, limit_ns)) atomicOr(err_flag, 1);  // phase 0 never completes
    mbar_inval(&bar);
  }
}

}  // namespace
}  // namespace kcv

extern "C" kleidicv_error_t kleidicv_gpu_selftest_bounded_wait(kleidicv_gpu_context_t *ctx,
                                                               uint64_t limit_ns) {
  if (!ctx) return KLEIDICV_ERROR_NULL_POINTER;
  if (limit_ns == 0 || limit_ns > 1000000000ull) return KLEIDICV_ERROR_RANGE;
  kcv::DeviceGuard guard(ctx->device);
  kcv::bounded_wait_selftest<<<1, 32, 0, ctx->stream>>>(ctx->d_err, limit_ns);
  return kcv::cuda_status(ctx, cudaGetLastError());
}
