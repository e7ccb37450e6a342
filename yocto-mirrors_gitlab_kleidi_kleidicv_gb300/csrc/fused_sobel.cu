#include "fused_inst.cuh"
namespace kcv {
bool launch_fused_sobel(const FilterJob &j, int *e, cudaStream_t s, cudaError_t *out, int *o,
                        const BatchLaunch *b) {
  if (j.ksize != 3) return false;
  switch (j.mode) {
    case MODE_SOBEL_X: return dispatch_channels<MODE_SOBEL_X, 3>(j, e, s, out, o, b);
    case MODE_SOBEL_Y: return dispatch_channels<MODE_SOBEL_Y, 3>(j, e, s, out, o, b);
  }
  return false;
}
}  // namespace kcv
