#include "fused_inst.cuh"
namespace kcv {
bool launch_fused_sigma_9(const FilterJob &j, int *e, cudaStream_t s, cudaError_t *out, int *o,
                        const BatchLaunch *b) {
  if (j.mode != MODE_SIGMA || j.ksize != 9) return false;
  return dispatch_channels<MODE_SIGMA, 9>(j, e, s, out, o, b);
}
}  // namespace kcv
