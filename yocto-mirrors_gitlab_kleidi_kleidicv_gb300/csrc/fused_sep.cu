#include "fused_inst.cuh"
namespace kcv {
bool launch_fused_sep(const FilterJob &j, int *e, cudaStream_t s, cudaError_t *out, int *o,
                        const BatchLaunch *b) {
  if (j.ksize != 5) return false;
  switch (j.mode) {
    case MODE_SEP_U8: return dispatch_channels<MODE_SEP_U8, 5>(j, e, s, out, o, b);
    case MODE_SEP_U16: return dispatch_channels<MODE_SEP_U16, 5>(j, e, s, out, o, b);
    case MODE_SEP_S16: return dispatch_channels<MODE_SEP_S16, 5>(j, e, s, out, o, b);
  }
  return false;
}
}  // namespace kcv
