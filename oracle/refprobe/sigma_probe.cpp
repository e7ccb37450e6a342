// Probe driver: runs the reference's own Gaussian half-kernel generator
// (kleidicv/include/kleidicv/filters/sigma.h, included from the reference
// tree) over a grid and prints one line per (kernel size, sigma):
//   <ksize> <sigma index> <ok> <w0> <w1> ... <w_half-1>
// sigma = float(index) / 100.0f for index in [0, 4000].
#include <cstdio>

#include "kleidicv/filters/sigma.h"

int main() {
  for (unsigned k = 3; k <= 255; k += 2) {
    const size_t half = kleidicv::get_half_kernel_size(k);
    for (int i = 0; i <= 4000; ++i) {
      const float sigma = static_cast<float>(i) / 100.0f;
      uint8_t hk[128] = {0};
      const bool ok = kleidicv::generate_gaussian_half_kernel(hk, half, sigma);
      std::printf("%u %d %d", k, i, ok ? 1 : 0);
      for (size_t j = 0; j < half; ++j) std::printf(" %u", ok ? hk[j] : 0u);
      std::printf("\n");
    }
  }
  return 0;
}
