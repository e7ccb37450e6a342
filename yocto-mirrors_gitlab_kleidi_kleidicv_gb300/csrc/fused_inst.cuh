// Helpers shared by the fused-kernel instantiation units.
#pragma once

#include "launch.h"
#include "sepfused.cuh"

namespace kcv {

template <int MODE, int K, int C>
cudaError_t launch_one(const FilterJob &job, int *err_flag, cudaStream_t stream) {
  const SmemLayout L = smem_layout<MODE>(job.threads, job.halo_chunks, job.box_lbw, job.stage_rows, job.stages);
  auto kern = sepfused_kernel<MODE, K, C>;
  static bool attr_set = false;  // per instantiation
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         200 * 1024);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  kern<<<dim3(job.strips, job.row_tiles), job.threads, L.total, stream>>>(job, err_flag);
  return cudaGetLastError();
}

template <int MODE, int K>
bool dispatch_channels(const FilterJob &job, int *err, cudaStream_t s, cudaError_t *out) {
  switch (job.channels) {
    case 1: *out = launch_one<MODE, K, 1>(job, err, s); return true;
    case 2: *out = launch_one<MODE, K, 2>(job, err, s); return true;
    case 3: *out = launch_one<MODE, K, 3>(job, err, s); return true;
    case 4: *out = launch_one<MODE, K, 4>(job, err, s); return true;
  }
  return false;
}

}  // namespace kcv
