// Probe driver: evaluates the reference's fixed-size border offset tables
// (kleidicv/include/kleidicv/workspace/border_{3x3,...,21x21}.h, included from
// the reference tree) and prints, for every kernel size, border type, extent n
// in [K-1, K+40] and index i in [0, n), the absolute source indices i + c_t:
//   <K> <border> <n> <i> <m_0> ... <m_{K-1}>
// border uses the C enum values (REPLICATE=1, REFLECT=2, WRAP=3, REVERSE=4).
#include <cstdio>

#include "kleidicv/workspace/border_15x15.h"
#include "kleidicv/workspace/border_21x21.h"
#include "kleidicv/workspace/border_3x3.h"
#include "kleidicv/workspace/border_5x5.h"
#include "kleidicv/workspace/border_7x7.h"
#include "kleidicv/workspace/border_9x9.h"

using kleidicv::FixedBorderInfo;
using kleidicv::FixedBorderType;

template <size_t K, typename Offsets>
static void collect(const Offsets &o, ptrdiff_t *c);

#define KCV_C(n) c[n] = o.c##n()
template <> void collect<3>(const FixedBorderInfo<uint8_t, 3>::Offsets &o, ptrdiff_t *c) { KCV_C(0); KCV_C(1); KCV_C(2); }
template <> void collect<5>(const FixedBorderInfo<uint8_t, 5>::Offsets &o, ptrdiff_t *c) { KCV_C(0); KCV_C(1); KCV_C(2); KCV_C(3); KCV_C(4); }
template <> void collect<7>(const FixedBorderInfo<uint8_t, 7>::Offsets &o, ptrdiff_t *c) { KCV_C(0); KCV_C(1); KCV_C(2); KCV_C(3); KCV_C(4); KCV_C(5); KCV_C(6); }
template <> void collect<9>(const FixedBorderInfo<uint8_t, 9>::Offsets &o, ptrdiff_t *c) { KCV_C(0); KCV_C(1); KCV_C(2); KCV_C(3); KCV_C(4); KCV_C(5); KCV_C(6); KCV_C(7); KCV_C(8); }
template <> void collect<15>(const FixedBorderInfo<uint8_t, 15>::Offsets &o, ptrdiff_t *c) {
  KCV_C(0); KCV_C(1); KCV_C(2); KCV_C(3); KCV_C(4); KCV_C(5); KCV_C(6); KCV_C(7); KCV_C(8); KCV_C(9); KCV_C(10); KCV_C(11); KCV_C(12); KCV_C(13); KCV_C(14);
}
template <> void collect<21>(const FixedBorderInfo<uint8_t, 21>::Offsets &o, ptrdiff_t *c) {
  KCV_C(0); KCV_C(1); KCV_C(2); KCV_C(3); KCV_C(4); KCV_C(5); KCV_C(6); KCV_C(7); KCV_C(8); KCV_C(9); KCV_C(10);
  KCV_C(11); KCV_C(12); KCV_C(13); KCV_C(14); KCV_C(15); KCV_C(16); KCV_C(17); KCV_C(18); KCV_C(19); KCV_C(20);
}

template <size_t K>
static void dump() {
  const struct { FixedBorderType t; int c_enum; } borders[] = {
      {FixedBorderType::REPLICATE, 1}, {FixedBorderType::REFLECT, 2},
      {FixedBorderType::WRAP, 3}, {FixedBorderType::REVERSE, 4}};
  for (const auto &b : borders) {
    for (size_t n = K - 1; n <= K + 40; ++n) {
      FixedBorderInfo<uint8_t, K> info{n, b.t};
      for (size_t i = 0; i < n; ++i) {
        ptrdiff_t c[K];
        collect<K>(info.offsets_with_border(i), c);
        std::printf("%zu %d %zu %zu", K, b.c_enum, n, i);
        for (size_t t = 0; t < K; ++t) std::printf(" %td", static_cast<ptrdiff_t>(i) + c[t]);
        std::printf("\n");
      }
    }
  }
}

int main() {
  dump<3>();
  dump<5>();
  dump<7>();
  dump<9>();
  dump<15>();
  dump<21>();
  return 0;
}
