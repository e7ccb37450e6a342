// Gaussian half-kernel generation on the host.
//
// Restates the algorithm of kleidicv/include/kleidicv/filters/sigma.h:27-79
// (float arithmetic, expf weights, normalisation to 256, rounding with error
// diffusion, "copy" when the centre weight rounds to 256).  This file is
// compiled with -ffp-contract=off so that no fused multiply-add changes the
// float rounding; the weights are checked byte-for-byte against the
// reference's own generator over k = 3..255 and sigma = 0..40 step 0.01.
#include <math.h>
#include <stddef.h>
#include <stdint.h>

#include "host.h"

namespace kcv {

bool gaussian_half_kernel(size_t ksize, float sigma, uint8_t *half) {
  const size_t mid = ksize / 2;  // index of the centre weight
  if (sigma == 0.0f) sigma = static_cast<float>(2 * mid + 1) * 0.15f + 0.35f;
  float gauss[128];
  const float coef = 1.0f / -(2.0f * sigma * sigma);
  float sum = 0.0f;
  for (size_t i = 0; i < mid; ++i) {
    const float d = static_cast<float>(mid - i);
    gauss[i] = expf(d * d * coef);
    sum += gauss[i];
  }
  const float scale = 256.0f / (sum * 2.0f + 1.0f);
  float carried = 0.0f;
  for (size_t i = 0; i < mid; ++i) {
    const float want = gauss[i] * scale - carried;
    const float got = roundf(want);
    half[i] = static_cast<uint8_t>(got);
    carried = got - want;
  }
  const unsigned centre = static_cast<uint16_t>(roundf(scale - carried));
  if (centre == 256u) return false;
  half[mid] = static_cast<uint8_t>(centre);
  return true;
}

}  // namespace kcv

extern "C" int kleidicv_gpu_gaussian_half_kernel(size_t kernel_size, float sigma,
                                                 uint8_t *half_kernel) {
  if (kernel_size < 3 || kernel_size > 255 || (kernel_size & 1) == 0 || !half_kernel) return 0;
  return kcv::gaussian_half_kernel(kernel_size, sigma, half_kernel) ? 1 : 0;
}
