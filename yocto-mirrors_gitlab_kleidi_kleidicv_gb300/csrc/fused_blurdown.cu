#include "fused_inst.cuh"
namespace kcv {
bool launch_fused_blurdown(const FilterJob &j, int *e, cudaStream_t s, cudaError_t *out, int *o,
                        const BatchLaunch *b) {
  if (j.mode != MODE_BLURDOWN) return false;
  return dispatch_channels<MODE_BLURDOWN, 5>(j, e, s, out, o, b);
}
size_t fused_smem_bytes(const FilterJob &job) {
  return smem_layout(job.mode, job.ksize, job.channels, job.threads, job.halo_chunks, job.box_lbw,
                     job.stage_rows, job.stages, job.use_tma != 0, job.border == BORDER_WRAP)
      .total;
}
static bool dispatch_fused(const FilterJob &job, int *err, cudaStream_t s, cudaError_t *out,
                           int *occ, const BatchLaunch *b) {
  return launch_fused_binom(job, err, s, out, occ, b) ||
         launch_fused_sigma_small(job, err, s, out, occ, b) ||
         launch_fused_sigma_9(job, err, s, out, occ, b) ||
         launch_fused_sigma_15(job, err, s, out, occ, b) ||
         launch_fused_sigma_21(job, err, s, out, occ, b) ||
         launch_fused_sep(job, err, s, out, occ, b) || launch_fused_blurdown(job, err, s, out, occ, b) ||
         launch_fused_sobel(job, err, s, out, occ, b);
}
cudaError_t launch_fused(const FilterJob &job, int *err, cudaStream_t s) {
  cudaError_t out = cudaErrorInvalidValue;
  return dispatch_fused(job, err, s, &out, nullptr, nullptr) ? out : cudaErrorInvalidValue;
}
int fused_blocks_per_sm(const FilterJob &job) {
  cudaError_t out = cudaErrorInvalidValue;
  int occ = 0;
  if (!dispatch_fused(job, nullptr, nullptr, &out, &occ, nullptr) || out != cudaSuccess) return 0;
  return occ;
}
cudaError_t launch_fused_batch(const FilterJob &rep, const BatchLaunch &b, int *err, cudaStream_t s) {
  cudaError_t out = cudaErrorInvalidValue;
  return dispatch_fused(rep, err, s, &out, nullptr, &b) ? out : cudaErrorInvalidValue;
}
int fused_batch_blocks_per_sm(const FilterJob &rep, const BatchLaunch &b) {
  cudaError_t out = cudaErrorInvalidValue;
  int occ = 0;
  if (!dispatch_fused(rep, nullptr, nullptr, &out, &occ, &b) || out != cudaSuccess) return 0;
  return occ;
}
}  // namespace kcv
