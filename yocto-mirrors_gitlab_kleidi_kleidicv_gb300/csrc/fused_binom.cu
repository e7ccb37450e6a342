#include "fused_inst.cuh"
namespace kcv {
bool launch_fused_binom(const FilterJob &j, int *e, cudaStream_t s, cudaError_t *out, int *o,
                        const BatchLaunch *b) {
  if (j.mode != MODE_BINOM) return false;
  switch (j.ksize) {
    case 3: return dispatch_channels<MODE_BINOM, 3>(j, e, s, out, o, b);
    case 5: return dispatch_channels<MODE_BINOM, 5>(j, e, s, out, o, b);
    case 7: return dispatch_channels<MODE_BINOM, 7>(j, e, s, out, o, b);
    case 9: return dispatch_channels<MODE_BINOM, 9>(j, e, s, out, o, b);
  }
  return false;
}
}  // namespace kcv
