// separable_filter_2d on one-channel 16-bit images with 5x5 kernels (sm_103a):
// the u16 entry point and the s16 extension.
//
// Arithmetic (kleidicv/src/filters/separable_filter_2d_neon.cpp:140-158 for
// u16): vertical sums of u16 x u16 products saturating at 2^32 - 1, then the
// horizontal sum of those times the horizontal taps, saturated to u16.  This
// kernel computes both passes in fp32, which gives the same outputs:
//  * u16: every product and partial sum is a non-negative integer.  While
//    they stay below 2^24 fp32 holds them exactly; a value that reaches 2^24
//    is rounded to a value that is still >= 2^24, and every later sum that
//    depends on it (taps >= 0; a zero tap contributes exactly 0) stays above
//    65535, as the reference's saturated result does.  So min(sum, 65535) is
//    exact whatever the taps;
//  * s16 (taps and data signed): the host routes a call here only when
//    32768 * sum|kx| * sum|ky| <= 2^24, so every product and partial sum of
//    both passes is an integer of magnitude <= 2^24, held exactly, and no
//    saturating s32 add of the reference can trigger.
// Both passes run on element pairs with the paired fp32 operations of sm_100+
// (__ffma2_rn: per component the same rounding as fmaf).  A lane's 8
// elements pair as (j, j + 4), so that a horizontal tap at distance d of
// pair j is the lane's own pair j + d wherever that lies in the lane; only
// the four pairs reaching into the neighbour lanes are assembled (one
// shuffle each).  Conversions avoid
// the slow integer<->float units: a 16-bit value v becomes
// the float 2^23 + v by placing its bits under the exponent of 2^23 (s16 is
// first biased by 2^15 with an xor), and a result r in [0, 65535] (u16, the
// horizontal sum starting at 2^23) or [-32768, 32767] (s16, + 1.5 * 2^23)
// keeps r in the low 16 bits of its float.
//
// A warp owns a strip of 32 lanes x 8 elements (16 bytes) of a row, of which
// lanes 1..30 produce output and lanes 0 and 31 only supply the two-element
// horizontal halo by shuffle, and a band of at most kSep16MaxBand destination
// rows.  It first requests every source row of the band at once (one 16-byte
// cp.async per lane and row into its own shared-memory slots: no register
// holds data in flight, and no other lane reads the slot), then streams down
// the band: the converted rows of the vertical window (five rows x 8 floats)
// rotate through statically indexed register slots (the row loop is unrolled
// by five), and each destination row costs one shared-memory load per lane.
// The source rows must be 16-byte aligned (the host copies larger unaligned
// sources into a 16-byte-row image first, and sends smaller ones to the
// tiled kernel of sepfused.cuh).  This pass reads only the lanes whose 8 elements lie
// inside the row, [0, wf) with wf = 8 * floor(w / 8), and stores only the
// outputs whose five columns lie inside that span, x in [2, wf - 2).  The
// other columns (x < 2 and x >= wf - 2) are edge elements, spread evenly over
// all items (each warp computes its share while its copies are in flight):
// one lane per (row, column), its 25 border-mapped source elements loaded
// independently, computed with the same operations.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cstdlib>

#include "launch.h"
#include "resident.cuh"
#include "sepfused.cuh"

namespace kcv {

namespace {

constexpr int kThreads16 = 128;
constexpr int kWarps16 = kThreads16 / 32;
constexpr int kLaneElems = 8;
constexpr int kStripElems = kSep16Lanes * kLaneElems;
constexpr int kStageRows = kSep16MaxBand + 4;          // source rows of a band
constexpr int kWarpStageBytes = kStageRows * 32 * 16;  // 9728
constexpr int kSmem16 = kWarps16 * kWarpStageBytes;    // 38912
constexpr int kGroups = (kStageRows + 4) / 5;          // copy groups of five rows: 4

// No "memory" clobber: nothing reads the slot before cp_async_wait, which
// carries it.
__device__ __forceinline__ void cp_async16(uint32_t dst, const void *src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Element pairs: x[j] = elements (j, j + 4) of the lane, so that the
// horizontal taps of a pair at distance d are the pair j + d whenever it lies
// in the lane (0 <= j + d <= 3).
template <bool S16>
__device__ __forceinline__ void to_float2(const uint4 &raw, float2 (&x)[kLaneElems / 2]) {
  constexpr float bias = S16 ? 8421376.0f : 8388608.0f;  // 2^23 (+ 2^15)
  const uint32_t w[4] = {raw.x, raw.y, raw.z, raw.w};  // w[i]: elements (2i, 2i + 1)
#pragma unroll
  for (int i = 0; i < 2; ++i) {
    const uint32_t a = S16 ? (w[i] ^ 0x80008000u) : w[i];          // elements 2i, 2i + 1
    const uint32_t b = S16 ? (w[i + 2] ^ 0x80008000u) : w[i + 2];  // elements 2i + 4, 2i + 5
    const float2 lo = make_float2(__uint_as_float(__byte_perm(a, 0x4B000000u, 0x7410)),
                                  __uint_as_float(__byte_perm(b, 0x4B000000u, 0x7410)));
    const float2 hi = make_float2(__uint_as_float(__byte_perm(a, 0x4B000000u, 0x7432)),
                                  __uint_as_float(__byte_perm(b, 0x4B000000u, 0x7432)));
    x[2 * i] = __fadd2_rn(lo, make_float2(-bias, -bias));
    x[2 * i + 1] = __fadd2_rn(hi, make_float2(-bias, -bias));
  }
}

// Horizontal pass of one element pair from its tap pairs (the taps of both
// elements, pair by pair); returns the two result words, each a float whose
// low 16 bits are the result.
template <bool S16>
__device__ __forceinline__ uint2 hfinish2(const float2 (&kx)[5], float2 a, float2 b, float2 c, float2 d,
                                             float2 e) {
  if constexpr (S16) {
    float2 acc = __fmul2_rn(kx[0], a);
    acc = __ffma2_rn(kx[1], b, acc);
    acc = __ffma2_rn(kx[2], c, acc);
    acc = __ffma2_rn(kx[3], d, acc);
    acc = __ffma2_rn(kx[4], e, acc);
    acc.x = fminf(fmaxf(acc.x, -32768.0f), 32767.0f);
    acc.y = fminf(fmaxf(acc.y, -32768.0f), 32767.0f);
    acc = __fadd2_rn(acc, make_float2(12582912.0f, 12582912.0f));  // 1.5 * 2^23 + r
    return make_uint2(__float_as_uint(acc.x), __float_as_uint(acc.y));
  } else {
    float2 acc = __ffma2_rn(kx[0], a, make_float2(8388608.0f, 8388608.0f));  // 2^23 + sum
    acc = __ffma2_rn(kx[1], b, acc);
    acc = __ffma2_rn(kx[2], c, acc);
    acc = __ffma2_rn(kx[3], d, acc);
    acc = __ffma2_rn(kx[4], e, acc);
    // 2^23 + min(sum, 65535)
    return make_uint2(__float_as_uint(fminf(acc.x, 8454143.0f)), __float_as_uint(fminf(acc.y, 8454143.0f)));
  }
}

// Destination row from the window slots (its source row y - 2 in slot S0,
// y - 1 in S0 + 1, ... modulo 5).
template <bool S16, int S0>
__device__ __forceinline__ uint4 filter_row(const float2 (&win)[5][kLaneElems / 2], const float2 (&kx)[5],
                                            const float2 (&ky)[5]) {
  // V[j]: vertical sums of elements (j, j + 4) of the lane.
  float2 V[4];
#pragma unroll
  for (int m = 0; m < 4; ++m) {
    float2 acc = __fmul2_rn(ky[0], win[S0 % 5][m]);
    acc = __ffma2_rn(ky[1], win[(S0 + 1) % 5][m], acc);
    acc = __ffma2_rn(ky[2], win[(S0 + 2) % 5][m], acc);
    acc = __ffma2_rn(ky[3], win[(S0 + 3) % 5][m], acc);
    V[m] = __ffma2_rn(ky[4], win[(S0 + 4) % 5][m], acc);
  }
  // The pairs at j + d = -2, -1 (elements -2, -1 are the left lane's 6, 7)
  // and j + d = 4, 5 (elements 8, 9 are the right lane's 0, 1).
  const float2 Cm2 = make_float2(__shfl_up_sync(0xffffffffu, V[2].y, 1), V[2].x);
  const float2 Cm1 = make_float2(__shfl_up_sync(0xffffffffu, V[3].y, 1), V[3].x);
  const float2 C4 = make_float2(V[0].y, __shfl_down_sync(0xffffffffu, V[0].x, 1));
  const float2 C5 = make_float2(V[1].y, __shfl_down_sync(0xffffffffu, V[1].x, 1));
  const uint2 h0 = hfinish2<S16>(kx, Cm2, Cm1, V[0], V[1], V[2]);
  const uint2 h1 = hfinish2<S16>(kx, Cm1, V[0], V[1], V[2], V[3]);
  const uint2 h2 = hfinish2<S16>(kx, V[0], V[1], V[2], V[3], C4);
  const uint2 h3 = hfinish2<S16>(kx, V[1], V[2], V[3], C4, C5);
  // Result j sits in the low 16 bits of h_j.x, result j + 4 in those of h_j.y.
  return make_uint4(__byte_perm(h0.x, h1.x, 0x5410), __byte_perm(h2.x, h3.x, 0x5410),
                    __byte_perm(h0.y, h1.y, 0x5410), __byte_perm(h2.y, h3.y, 0x5410));
}

__host__ __device__ inline int full_span(int w) { return w / kLaneElems * kLaneElems; }

// Edge columns: x < 2 and x >= max(2, wf - 2), inside the row.
__host__ __device__ inline int edge_left(int w) { return w < 2 ? w : 2; }
__host__ __device__ inline int edge_right_start(int w) {
  const int r = full_span(w) - 2;
  return r > edge_left(w) ? r : edge_left(w);
}
__host__ __device__ inline int edge_cols(int w) { return edge_left(w) + (w - edge_right_start(w)); }

// Edge element: destination (y, x) from its 25 border-mapped source
// elements, with the operations of filter_row.
template <bool S16>
__device__ __forceinline__ void edge_element16(const Sep16Job &j, int y, int x) {
  const uint32_t bv = static_cast<uint32_t>(j.border_value) & 0xFFFFu;
  const uint16_t *rows[5];
  int cols[5];
#pragma unroll
  for (int d = 0; d < 5; ++d) {
    const int my = map_index(y + d - 2, j.h, j.border);
    rows[d] = my < 0 ? nullptr : reinterpret_cast<const uint16_t *>(j.src + static_cast<int64_t>(my) * j.src_stride);
    cols[d] = map_index(x + d - 2, j.w, j.border);
  }
  uint32_t raw[5][5];
#pragma unroll
  for (int r = 0; r < 5; ++r)
#pragma unroll
    for (int c = 0; c < 5; ++c) raw[r][c] = (rows[r] && cols[c] >= 0) ? __ldg(rows[r] + cols[c]) : bv;
  float2 kx[5];
#pragma unroll
  for (int t = 0; t < 5; ++t) kx[t] = make_float2(j.kx[t], j.kx[t]);
  float V[5];
#pragma unroll
  for (int c = 0; c < 5; ++c) {
    float x5[5];
#pragma unroll
    for (int r = 0; r < 5; ++r) {
      const uint32_t v = S16 ? (raw[r][c] ^ 0x8000u) : raw[r][c];
      x5[r] = __uint_as_float(v | 0x4B000000u) - (S16 ? 8421376.0f : 8388608.0f);
    }
    float acc = j.ky[0] * x5[0];
    acc = fmaf(j.ky[1], x5[1], acc);
    acc = fmaf(j.ky[2], x5[2], acc);
    acc = fmaf(j.ky[3], x5[3], acc);
    V[c] = fmaf(j.ky[4], x5[4], acc);
  }
  // The pair form with the element in both halves.
  const uint32_t bits = hfinish2<S16>(kx, make_float2(V[0], V[0]), make_float2(V[1], V[1]), make_float2(V[2], V[2]),
                                      make_float2(V[3], V[3]), make_float2(V[4], V[4])).x;
  reinterpret_cast<uint16_t *>(j.dst + static_cast<int64_t>(y) * j.dst_stride)[x] = static_cast<uint16_t>(bits);
}

template <bool S16, bool SIMPLE>
__device__ __forceinline__ void band_loop16(const Sep16Job &j, const uint4 *stage, int lane, int rows, uint8_t *d,
                                            long e0, int wf, bool outputs, bool full_store);

template <bool S16>
__device__ __forceinline__ void run_band16(const Sep16Job &j, uint4 *stage, int strip, int band, int lane) {
  const long e0 = static_cast<long>(strip) * kStripElems + kLaneElems * lane - kLaneElems;
  const int wf = full_span(j.w);
  const bool fast = e0 >= 0 && e0 + kLaneElems <= wf;
  // Outputs x in [2, wf - 2) of lanes 1..30.
  const bool outputs = lane >= 1 && lane <= kSep16Lanes && e0 + kLaneElems > 2 && e0 < wf - 2;
  const bool full_store =
      outputs && e0 >= 2 && e0 + kLaneElems <= wf - 2 &&
      ((reinterpret_cast<uintptr_t>(j.dst) | static_cast<uintptr_t>(j.dst_stride)) & 15) == 0;
  const uint32_t bv2 = (static_cast<uint32_t>(j.border_value) & 0xFFFFu) * 0x00010001u;

  // Band b has band_q + (b < band_r) rows (at most kSep16MaxBand).
  const int rows = j.band_q + (band < j.band_r ? 1 : 0);
  const int y0 = band * j.band_q + min(band, j.band_r);
  const int y1 = y0 + rows;
  const int nrows = rows + 4;  // source rows y0 - 2 .. y1 + 1
  static_assert(kGroups == 4, "the waits below assume four copy groups");
  // Request every source row: slot rr of the lane holds row y0 - 2 + rr, in
  // kGroups copy groups of five rows (rows [5g, 5g + 5); empty groups at the
  // end), so that the rows are filtered as their group lands.
  const uint32_t sbase = static_cast<uint32_t>(__cvta_generic_to_shared(stage + lane));
  if (fast && y0 >= 2 && y1 + 2 <= j.h) {
    // Rows inside the image: consecutive.
    const uint8_t *g = j.src + static_cast<int64_t>(y0 - 2) * j.src_stride + 2 * e0;
    uint32_t a = sbase;
    int rr = 0;
#pragma unroll
    for (int grp = 0; grp < kGroups; ++grp) {
#pragma unroll 1
      for (; rr < min(nrows, 5 * grp + 5); ++rr, a += 32 * 16, g += j.src_stride) cp_async16(a, g);
      cp_async_commit();
    }
  } else {
    int rr = 0;
#pragma unroll
    for (int grp = 0; grp < kGroups; ++grp) {
#pragma unroll 1
      for (; rr < min(nrows, 5 * grp + 5); ++rr) {
        const int y = map_index(y0 - 2 + rr, j.h, j.border);
        if (y >= 0 && fast) {
          cp_async16(sbase + rr * 32 * 16, j.src + static_cast<int64_t>(y) * j.src_stride + 2 * e0);
        } else {
          // A CONSTANT border row, or a lane outside the span (its elements
          // are read by no stored output).
          stage[rr * 32 + lane] = y < 0 ? make_uint4(bv2, bv2, bv2, bv2) : make_uint4(0u, 0u, 0u, 0u);
        }
      }
      cp_async_commit();
    }
  }
  // Edge elements (row-major over the edge columns of every row) go in
  // passes of 32, one lane each, to every edge_every-th item, edge_per
  // passes each: a few full-width passes per SM, computed while the item's
  // copies are in flight.
  {
    const int t = band * j.strips + strip;
    if (t % j.edge_every == 0) {
      const int ne = edge_cols(j.w), nl = edge_left(j.w), rs = edge_right_start(j.w);
      const int total = ne * j.h;
      const int p0 = t / j.edge_every * j.edge_per;
      for (int p = p0; p < p0 + j.edge_per; ++p) {
        const int k = p * 32 + lane;
        if (k < total) {
          const int y = k / ne, i = k - y * ne;
          edge_element16<S16>(j, y, i < nl ? i : rs + (i - nl));
        }
      }
    }
  }

  uint8_t *d = j.dst + static_cast<int64_t>(y0) * j.dst_stride + 2 * e0;
  // The byte-store path only where some lane of the warp needs it.
  if (__all_sync(0xffffffffu, !outputs || full_store))
    band_loop16<S16, true>(j, stage, lane, rows, d, e0, wf, outputs, full_store);
  else
    band_loop16<S16, false>(j, stage, lane, rows, d, e0, wf, outputs, full_store);
}

template <bool S16, bool SIMPLE>
__device__ __forceinline__ void band_loop16(const Sep16Job &j, const uint4 *stage, int lane, int rows, uint8_t *d,
                                            long e0, int wf, bool outputs, bool full_store) {
  float2 kx[5], ky[5];
#pragma unroll
  for (int t = 0; t < 5; ++t) {
    kx[t] = make_float2(j.kx[t], j.kx[t]);
    ky[t] = make_float2(j.ky[t], j.ky[t]);
  }
  // Window slot k holds the converted source row rr with rr = k mod 5.
  float2 win[5][kLaneElems / 2];
  cp_async_wait<kGroups - 1>();  // group 0: rows 0 .. 4
#pragma unroll
  for (int rr = 0; rr < 4; ++rr) to_float2<S16>(stage[rr * 32 + lane], win[rr]);
#pragma unroll 1
  for (int base = 0; base < rows; base += 5) {
    // Destination rows base .. base + 4 read source rows up to base + 8:
    // groups up to base / 5 + 1.
    switch (base / 5) {
      case 0: cp_async_wait<kGroups - 2>(); break;
      case 1: cp_async_wait<kGroups - 3>(); break;
      default: cp_async_wait<0>(); break;
    }
    static_for<0, 5>([&](auto sc) {
      constexpr int S = decltype(sc)::value;
      constexpr int slot = (S + 4) % 5;  // receives source row rr = base + S + 4
      if (base + S >= rows) return;  // past the band (the loop ends here)
      to_float2<S16>(stage[(base + S + 4) * 32 + lane], win[slot]);
      const uint4 out = filter_row<S16, S>(win, kx, ky);
      if (SIMPLE) {
        if (outputs) *reinterpret_cast<uint4 *>(d) = out;
      } else if (outputs) {
        if (full_store) {
          *reinterpret_cast<uint4 *>(d) = out;
        } else {
          const uint32_t o[4] = {out.x, out.y, out.z, out.w};
          uint16_t *d16 = reinterpret_cast<uint16_t *>(d);
#pragma unroll
          for (int k = 0; k < kLaneElems; ++k)
            if (e0 + k >= 2 && e0 + k < wf - 2) d16[k] = static_cast<uint16_t>(o[k >> 1] >> (16 * (k & 1)));
        }
      }
      d += j.dst_stride;
    });
  }
}

template <bool S16>
__global__ void __launch_bounds__(kThreads16, 5) sep16_kernel(const __grid_constant__ Sep16Job j) {
  extern __shared__ __align__(16) uint4 stage16[];
  // The next call on the stream may start its CTAs as ours finish; it reads
  // nothing before this grid has completed.
  launch_dependents();
  grid_dependency_wait();  // the source may be the previous call's output
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint4 *stage = stage16 + warp * (kWarpStageBytes / 16);
  // Items go round the CTAs first, so that every SM (the grid is whole
  // waves of resident CTAs) gets the same number.
  const int gw = warp * gridDim.x + blockIdx.x;
  const int nw = gridDim.x * kWarps16;
  const int items = j.strips * j.bands;
  for (int t = gw; t < items; t += nw) {
    // Strips rotate by 7 per band: a warp's items do not all land on the
    // costlier strips at the row's ends.
    const int band = t / j.strips, q = t - band * j.strips;
    const int strip = static_cast<int>((q + 7L * band) % j.strips);
    run_band16<S16>(j, stage, strip, band, lane);
  }
}

template <bool S16>
cudaError_t launch16(Sep16Job &j, int sm_count, cudaStream_t stream) {
  auto kern = sep16_kernel<S16>;
  int occ = 0;
  const cudaError_t err = resident_ctas_per_sm<sep16_kernel<S16>>(kThreads16, kSmem16, &occ);
  if (err != cudaSuccess) return err;
  const long resident = static_cast<long>(occ) * std::max(sm_count, 1);
  const long slots = resident * kWarps16;
  j.strips = (j.w + kStripElems - 1) / kStripElems;
  // Bands of at most kSep16MaxBand rows, as many as give every resident warp
  // the same number of items (one wave of n items per warp).
  const long min_bands = (j.h + kSep16MaxBand - 1) / kSep16MaxBand;
  const long per_warp = std::max(1L, (min_bands * j.strips + slots - 1) / slots);
  j.bands = static_cast<int32_t>(std::min<long>(j.h, std::max(min_bands, per_warp * slots / j.strips)));
  j.band_q = j.h / j.bands;
  j.band_r = j.h % j.bands;
  const long items = static_cast<long>(j.strips) * j.bands;
  const long passes = (static_cast<long>(edge_cols(j.w)) * j.h + 31) / 32;
  j.edge_every = static_cast<int32_t>(passes <= items ? items / std::max(passes, 1L) : 1);
  j.edge_per = static_cast<int32_t>(passes <= items ? 1 : (passes + items - 1) / items);
  const long grid = std::max(1L, std::min(resident, (items + kWarps16 - 1) / kWarps16));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(static_cast<unsigned>(grid));
  cfg.blockDim = dim3(kThreads16);
  cfg.dynamicSmemBytes = kSmem16;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, j);
}

}  // namespace

bool sep16_eligible(const FilterJob &f) {
  if ((f.mode != MODE_SEP_U16 && f.mode != MODE_SEP_S16) || f.ksize != 5 || f.channels != 1) return false;
  // 16-byte copies of source rows; 16-bit destination stores.
  if (((reinterpret_cast<uintptr_t>(f.src) | static_cast<uintptr_t>(f.src_stride)) & 15) != 0) return false;
  if (((reinterpret_cast<uintptr_t>(f.dst) | static_cast<uintptr_t>(f.dst_stride)) & 1) != 0) return false;
  // Item and edge indices in 32 bits.
  if (static_cast<long>(f.height) * (f.width / kStripElems + 1) >= (1L << 30) ||
      static_cast<long>(f.height) * 16 >= (1L << 30))
    return false;
  if (f.mode == MODE_SEP_U16) return true;
  long sx = 0, sy = 0;
  for (int t = 0; t < 5; ++t) {
    sx += std::abs(static_cast<long>(f.wx[t]));
    sy += std::abs(static_cast<long>(f.wy[t]));
  }
  return 32768L * sx * sy <= (1L << 24);
}

cudaError_t launch_sep16(const FilterJob &f, int sm_count, cudaStream_t stream) {
  Sep16Job j{};
  j.src = f.src;
  j.dst = f.dst;
  j.src_stride = f.src_stride;
  j.dst_stride = f.dst_stride;
  j.w = f.width;
  j.h = f.height;
  j.border = f.border;
  j.border_value = f.border_value;
  for (int t = 0; t < 5; ++t) {
    j.kx[t] = static_cast<float>(f.wx[t]);
    j.ky[t] = static_cast<float>(f.wy[t]);
  }
  return f.mode == MODE_SEP_S16 ? launch16<true>(j, sm_count, stream) : launch16<false>(j, sm_count, stream);
}

}  // namespace kcv
