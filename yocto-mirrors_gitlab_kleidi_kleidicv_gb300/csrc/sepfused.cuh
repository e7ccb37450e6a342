// Fused row-streaming separable stencil for sm_103a.
//
// One CTA owns a vertical strip of the image (threads x 16-byte chunks of a
// row, the outer HC chunks on each side being the horizontal filter halo)
// and walks down a band of rows:
//
//   * rows reach shared memory through a ring of TMA stages
//     (cp.async.bulk.tensor.2d + mbarrier transaction counts) whenever the
//     source is 16-byte aligned.  The border is resolved in the address
//     calculation, never by a padded copy: a stage that reaches above or
//     below the image loads the border-mapped source rows as single-row
//     boxes, a WRAP border on an edge strip adds one box from the far end of
//     the row, and chunks hanging over the left/right edge gather their
//     mapped elements from shared memory.  Sources that TMA cannot address
//     (unaligned base or stride) are read with plain loads instead;
//   * output rows are produced in blocks of M: each thread reads the M+K-1
//     source rows of its chunk from the ring once, unpacks each once (u8 as
//     packed 16-bit lanes) and adds it into the M vertical sums it belongs
//     to, in the reference's intermediate width and rounding;
//   * the horizontal pass then takes one output row at a time and reads the
//     neighbouring lanes' vertical results at compile-time offsets (tap
//     distance = channels elements): by warp shuffle straight from their
//     registers when the halo is at most six words per lane array, otherwise
//     through the warp's two shared V rows; the result is stored with
//     16-byte stores (32-byte for the Sobel derivatives).
//
// Every output byte equals the reference's: the arithmetic per mode follows
// kleidicv/src/filters/gaussian_blur_fixed_neon.cpp (binomial 3/5/7/9 and
// generated-sigma kernels), separable_filter_2d_neon.cpp (u8/u16 saturation)
// blur_and_downsample_neon.cpp and sobel_neon.cpp (3x3 derivatives, u8 in,
// s16 out: 32 destination bytes per chunk), with the border offset tables of
// kleidicv/include/kleidicv/workspace/border_*.h restated as a single-fold
// index map.
#pragma once

#include <stdint.h>

#include <type_traits>
#include <utility>

#include "kcv_job.h"
#include "ptx.cuh"

namespace kcv {

// ---------------------------------------------------------------------------
// Compile-time loop: calls f(std::integral_constant<int, I>) for I in [B, E).
template <int B, int E, typename F>
__device__ __forceinline__ void static_for(F &&f) {
  if constexpr (B < E) {
    f(std::integral_constant<int, B>{});
    static_for<B + 1, E>(f);
  }
}

constexpr int floor_div(int a, int b) { return a >= 0 ? a / b : -((-a + b - 1) / b); }

template <int MODE>
struct ModeTraits {
  static constexpr int ES = (MODE == MODE_SEP_U16 || MODE == MODE_SEP_S16) ? 2 : 1;
  static constexpr bool LANES = ES == 1;  // u8 data held as packed 16-bit lanes
  static constexpr bool SOBEL = MODE == MODE_SOBEL_X || MODE == MODE_SOBEL_Y;
  // Destination bytes per source byte: the Sobel derivatives widen u8 to s16.
  static constexpr int OSCALE = SOBEL ? 2 : 1;
};

template <int MODE, int K, int C>
struct Geo {
  static constexpr int R = K / 2;
  static constexpr int ES = ModeTraits<MODE>::ES;
  static constexpr int HALO_ELEMS = MODE == MODE_BLURDOWN ? 2 * C + 2 : R * C;
  static constexpr int HC = (HALO_ELEMS * ES + kChunk - 1) / kChunk;  // halo chunks / side
  static constexpr int HW = 4 * HC;                                   // halo words / side
  static constexpr int NW = 4 + 2 * HW;  // 32-bit words read around a chunk
};

// ---------------------------------------------------------------------------
// Border map (single fold; exact for n >= K - 1).  Positions that are farther
// than one fold from the image are only ever read by halo lanes whose results
// are discarded, so they are clamped to stay inside the allocation.
__device__ __forceinline__ int map_index(int i, int n, int border) {
  if (static_cast<unsigned>(i) < static_cast<unsigned>(n)) return i;
  int m;
  switch (border) {
    case BORDER_REPLICATE: m = i < 0 ? 0 : n - 1; break;
    case BORDER_REFLECT: m = i < 0 ? -i - 1 : 2 * n - i - 1; break;
    case BORDER_WRAP: m = i < 0 ? i + n : i - n; break;
    case BORDER_REVERSE: m = i < 0 ? -i : 2 * n - i - 2; break;
    default: return -1;  // CONSTANT
  }
  return m < 0 ? 0 : (m >= n ? n - 1 : m);
}

// Loads the in-image 16 bytes of a row at byte offset xb (0 <= xb, xb + 16 <=
// row bytes) with 16-byte loads: directly when aligned, otherwise from the two
// aligned blocks covering it when both lie inside the row.  Returns false when
// neither applies (the caller then assembles the chunk element by element).
__device__ __forceinline__ bool load_chunk_fast(const uint8_t *row, long xb, long wcb, uint4 &out) {
  const uint8_t *p = row + xb;
  const uintptr_t pa = reinterpret_cast<uintptr_t>(p);
  if ((pa & 15) == 0) {
    out = ld_nc_v4(p);
    return true;
  }
  const uint8_t *a = reinterpret_cast<const uint8_t *>(pa & ~static_cast<uintptr_t>(15));
  if (a < row || a + 32 > row + wcb) return false;
  const uint4 u = ld_nc_v4(a), v = ld_nc_v4(a + 16);
  const uint32_t w[8] = {u.x, u.y, u.z, u.w, v.x, v.y, v.z, v.w};
  const int sh = static_cast<int>(pa & 15), q = sh >> 2, s8 = (sh & 3) * 8;
  uint32_t o[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const uint32_t lo = q == 0 ? w[k] : q == 1 ? w[k + 1] : q == 2 ? w[k + 2] : w[k + 3];
    const uint32_t hi = q == 0 ? w[k + 1] : q == 1 ? w[k + 2] : q == 2 ? w[k + 3] : w[k + 4];
    o[k] = __funnelshift_r(lo, hi, s8);
  }
  out = make_uint4(o[0], o[1], o[2], o[3]);
  return true;
}

// Stores a lane's 16 result bytes `r` at `d`, which lies m = d % 16 bytes past
// a 16-byte boundary, as the aligned block [d - m, d + 16 - m): its first m
// bytes are the last m of the previous lane's result `pr`.  The first lane
// of a run (its previous lane stores nothing) writes bytes [0, 16 - m) of
// its own result instead, and the last lane (its next lane stores nothing)
// also writes bytes [16 - m, 16), which no block covers.
__device__ __forceinline__ void store_shifted(uint8_t *d, const uint4 &pr, const uint4 &r, bool first, bool last) {
  const int m = static_cast<int>(reinterpret_cast<uintptr_t>(d) & 15);
  if (m == 0) {
    *reinterpret_cast<uint4 *>(d) = r;
    return;
  }
  if (!first) {
    // Bytes [16 - m, 32 - m) of pr : r.
    const uint32_t c[8] = {pr.x, pr.y, pr.z, pr.w, r.x, r.y, r.z, r.w};
    const int s = 16 - m, q = s >> 2, s8 = (s & 3) * 8;
    uint32_t o[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const uint32_t lo = q == 0 ? c[k] : q == 1 ? c[k + 1] : q == 2 ? c[k + 2] : c[k + 3];
      const uint32_t hi = q == 0 ? c[k + 1] : q == 1 ? c[k + 2] : q == 2 ? c[k + 3] : c[k + 4];
      o[k] = __funnelshift_r(lo, hi, s8);
    }
    *reinterpret_cast<uint4 *>(d - m) = make_uint4(o[0], o[1], o[2], o[3]);
  }
  if (first || last) {
    const uint32_t w[4] = {r.x, r.y, r.z, r.w};
#pragma unroll
    for (int i = 0; i < 16; ++i)
      if (i < 16 - m ? first : last) d[i] = static_cast<uint8_t>(w[i >> 2] >> (8 * (i & 3)));
  }
}

// Where the bytes of the tile rows live in shared memory.  The ring holds
// ring_rows = stages * stage_rows rows; stage s of a tile occupies ring rows
// [slot * stage_rows, slot * stage_rows + stage_rows) with slot = (g + s) mod
// stages, so tile row q (global stage counter g) is ring row
// (g * stage_rows + q) mod ring_rows.  With TMA the span is laid out as
// [box][ring row][box bytes] (every box of a stage-rows-high TMA copy lands
// on consecutive ring rows), the two wrap areas as [area][ring row][256 B].
struct RingGeo {
  long xs;        // first byte of the span (multiple of 16, may be negative)
  long span_end;  // xs + boxes * box bytes
  long wcb;       // bytes per image row
  long wrapl_x;   // first byte of the left wrap area's box (valid if wrap_left)
  int lbw;        // log2 of the span box width in bytes (256 or 2048)
  int ring_rows;  // rows in the ring (power of two)
  bool wrap_left, wrap_right;
};

// Byte `b` (absolute offset within the image row) of ring row `rr`, from the
// span or a wrap area.  Bytes that were not staged read as 0; only halo lanes
// whose results are discarded can ask for them.
__device__ __forceinline__ uint32_t staged_byte(const uint8_t *ring, const uint8_t *wrap,
                                                const RingGeo &g, int rr, long b) {
  const int bw = 1 << g.lbw;
  if (b >= g.xs && b < g.span_end) {
    const int o = static_cast<int>(b - g.xs);
    return ring[(o >> g.lbw) * g.ring_rows * bw + rr * bw + (o & (bw - 1))];
  }
  if (g.wrap_left && b >= g.wrapl_x && b < g.wrapl_x + 256) return wrap[rr * 256 + (b - g.wrapl_x)];
  if (g.wrap_right && b >= 0 && b < 256) return wrap[(g.ring_rows + rr) * 256 + b];
  return 0;
}

// ---------------------------------------------------------------------------
// Binomial coefficient sets and rounding shifts of the reference
// (gaussian_blur_fixed_neon.cpp: 3x3 :27-85, 5x5 :87-153, 7x7 :155-281,
// 9x9 :283-459).
template <int K>
struct Binomial;
template <>
struct Binomial<3> {
  __host__ __device__ static constexpr int c(int i) { return i == 1 ? 2 : 1; }
  static constexpr int shift = 4;
};
template <>
struct Binomial<5> {
  __host__ __device__ static constexpr int c(int i) {
    return i == 2 ? 6 : (i == 1 || i == 3) ? 4 : 1;
  }
  static constexpr int shift = 8;
};
template <>
struct Binomial<7> {
  __host__ __device__ static constexpr int c(int i) {
    return i == 3 ? 18 : (i == 2 || i == 4) ? 14 : (i == 1 || i == 5) ? 7 : 2;
  }
  static constexpr int shift = 12;
};
template <>
struct Binomial<9> {
  __host__ __device__ static constexpr int c(int i) {
    return i == 4 ? 60 : (i == 3 || i == 5) ? 51 : (i == 2 || i == 6) ? 30
           : (i == 1 || i == 7) ? 13 : 4;
  }
  static constexpr int shift = 16;
};

// Taps held in registers for the duration of a tile.  Gaussian kernels are
// symmetric: y[0..K/2] only, used in both directions.
struct Taps {
  uint32_t y[kMaxTaps];
  uint32_t x[kMaxTaps];
};

// ---------------------------------------------------------------------------
// A row chunk (16 bytes) in arithmetic form: u8 data as eight words of two
// 16-bit lanes (x[0..3] = elements 4i, 4i+2; x[4..7] = elements 4i+1, 4i+3),
// u16 as eight u32, s16 as eight sign-extended s32.
template <int MODE>
__device__ __forceinline__ void unpack_chunk(const uint4 &raw, uint32_t (&x)[8]) {
  const uint32_t w[4] = {raw.x, raw.y, raw.z, raw.w};
  if constexpr (ModeTraits<MODE>::LANES) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      x[i] = w[i] & 0x00FF00FFu;
      x[4 + i] = __byte_perm(w[i], 0u, 0x4341);
    }
  } else if constexpr (MODE == MODE_SEP_U16) {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      x[2 * i] = w[i] & 0xFFFFu;
      x[2 * i + 1] = w[i] >> 16;
    }
  } else {
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      x[2 * i] = static_cast<uint32_t>(static_cast<int32_t>(static_cast<int16_t>(w[i] & 0xFFFFu)));
      x[2 * i + 1] = static_cast<uint32_t>(static_cast<int32_t>(w[i]) >> 16);
    }
  }
}

// One vertical tap: acc + weight(T) * x in the mode's intermediate arithmetic.
template <int MODE, int K, bool NARROW, int T>
__device__ __forceinline__ uint32_t vtap(uint32_t acc, uint32_t x, const Taps &tp) {
  if constexpr (MODE == MODE_SIGMA) {
    constexpr int H = T <= K / 2 ? T : K - 1 - T;
    return acc + tp.y[H] * x;  // weights sum to 256: 16-bit lanes never carry
  } else if constexpr (MODE == MODE_BINOM) {
    return acc + static_cast<uint32_t>(Binomial<K>::c(T)) * x;  // <= 255 * 256
  } else if constexpr (MODE == MODE_BLURDOWN) {
    return acc + static_cast<uint32_t>(Binomial<5>::c(T)) * x;
  } else if constexpr (MODE == MODE_SOBEL_X) {
    // [1 2 1] (sobel_neon.cpp:33-45): lanes <= 1020.
    return T == 1 ? acc + 2u * x : acc + x;
  } else if constexpr (MODE == MODE_SOBEL_Y) {
    // [-1 0 1] (sobel_neon.cpp:92-101), on lanes biased by +256 so that the
    // difference stays inside its 16-bit lane: lanes in [1, 511].
    return T == 0 ? acc - x : (T == 2 ? acc + x : acc);
  } else if constexpr (MODE == MODE_SEP_U8) {
    // Saturating u16 in the reference (separable_filter_2d_neon.cpp:38-56).
    // Taps are non-negative, so any lane reaching 255 forces a 255 output:
    // clamping products and sum to 255 gives the same bytes; with NARROW taps
    // (sum <= 257) the plain lane sum cannot carry.
    if constexpr (NARROW) return acc + tp.y[T] * x;
    else return acc + vmin_u16x2(tp.y[T] * x, 0x00FF00FFu);
  } else if constexpr (MODE == MODE_SEP_U16) {
    // separable_filter_2d_neon.cpp:140-158: saturating u32 sums of u16 x u16
    // products, then a saturating narrow of the horizontal sum; clamping each
    // product and the sum to 65535 yields the same outputs (taps >= 0).
    if constexpr (NARROW) return acc + tp.y[T] * x;
    else return acc + min(tp.y[T] * x, 0xFFFFu);
  } else {
    // s16 extension: saturating s32 adds in tap order.
    const int32_t p = static_cast<int32_t>(tp.y[T]) * static_cast<int32_t>(x);
    if constexpr (NARROW) return static_cast<uint32_t>(static_cast<int32_t>(acc) + p);
    else return static_cast<uint32_t>(add_sat_s32(static_cast<int32_t>(acc), p));
  }
}

template <int MODE>
__device__ __forceinline__ uint32_t vfinish(uint32_t acc) {
  if constexpr (MODE == MODE_SIGMA) return __byte_perm(acc, 0u, 0x4341);  // (acc >> 8) per lane
  else if constexpr (MODE == MODE_SEP_U8) return vmin_u16x2(acc, 0x00FF00FFu);
  else if constexpr (MODE == MODE_SEP_U16) return min(acc, 0xFFFFu);
  else return acc;  // binomial / blur-and-downsample (exact), s16 (s32 bits)
}

// Vertical pass of one block: block_out_rows output rows from
// block_in_rows consecutive ring rows starting at ring row rr0 (modulo
// ring_rows).  Each source
// row is read from shared memory and unpacked once, then added into every
// output row it belongs to (taps outer, lanes inner: independent chains).
template <int MODE, int K, bool NARROW>
__device__ __forceinline__ void vertical_block(const uint8_t *lane_base, uint32_t pitch,
                                               uint32_t rr0, uint32_t ring_rows, const Taps &tp,
                                               uint32_t (&v)[block_out_rows(MODE, K)][8]) {
  constexpr int M = block_out_rows(MODE, K);
  constexpr int NIN = block_in_rows(MODE, K);
  constexpr int KT = MODE == MODE_BLURDOWN ? 5 : K;
  uint32_t acc[M][8];
  static_for<0, M>([&](auto mc) {
    constexpr int Mi = decltype(mc)::value;
#pragma unroll
    for (int j = 0; j < 8; ++j)
      acc[Mi][j] = MODE == MODE_SIGMA ? 0x00800080u : (MODE == MODE_SOBEL_Y ? 0x01000100u : 0u);
  });
  static_for<0, NIN>([&](auto ic) {
    constexpr int I = decltype(ic)::value;
    uint32_t rr = rr0 + I;  // rr0 < ring_rows and I < ring_rows: one wrap at most
    if (rr >= ring_rows) rr -= ring_rows;
    const uint4 raw = *reinterpret_cast<const uint4 *>(lane_base + rr * pitch);
    uint32_t x[8];
    unpack_chunk<MODE>(raw, x);
    static_for<0, M>([&](auto mc) {
      constexpr int Mi = decltype(mc)::value;
      constexpr int T = MODE == MODE_BLURDOWN ? I - 2 * Mi : I - Mi;
      if constexpr (T >= 0 && T < KT) {
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[Mi][j] = vtap<MODE, K, NARROW, T>(acc[Mi][j], x[j], tp);
      }
    });
  });
  static_for<0, M>([&](auto mc) {
    constexpr int Mi = decltype(mc)::value;
#pragma unroll
    for (int j = 0; j < 8; ++j) v[Mi][j] = vfinish<MODE>(acc[Mi][j]);
  });
}

// ---------------------------------------------------------------------------
// Horizontal pass helpers for the lane form.  lo/hi hold NW words around the
// thread's own 4 words (which start at index HW).  Returns the pair of lanes
// for elements (4*I + P + D, 4*I + P + D + 2) of the thread's span.
template <int HW, int NW, int I, int P, int D>
__device__ __forceinline__ uint32_t pair_at(const uint32_t (&lo)[NW], const uint32_t (&hi)[NW]) {
  constexpr int g = P + D;
  constexpr int q = floor_div(g, 4);
  constexpr int rem = g - 4 * q;
  constexpr int w = HW + I + q;
  static_assert(w >= 0 && w + (rem >= 2 ? 1 : 0) < NW, "halo too small");
  if constexpr ((rem & 1) == 0) {
    if constexpr (rem < 2) return lo[w];
    else return __byte_perm(lo[w], lo[w + 1], 0x5432);
  } else {
    if constexpr (rem < 2) return hi[w];
    else return __byte_perm(hi[w], hi[w + 1], 0x5432);
  }
}

// The words of a lane array that the lane-form horizontal pass reads,
// relative to the lane's own first word: [first(), last()] (pair_at's word
// w - HW, plus w + 1 - HW for pairs straddling two words).
__host__ __device__ constexpr int lane_span_first(int k, int c) {
  int m = 0;
  for (int d = -(k / 2); d <= k / 2; ++d)
    for (int p = 0; p < 2; ++p) m = floor_div(p + d * c, 4) < m ? floor_div(p + d * c, 4) : m;
  return m;
}
__host__ __device__ constexpr int lane_span_last(int k, int c) {
  int m = 3;
  for (int d = -(k / 2); d <= k / 2; ++d)
    for (int p = 0; p < 2; ++p) {
      const int g = p + d * c, q = floor_div(g, 4), w = 3 + q + (g - 4 * q >= 2 ? 1 : 0);
      m = w > m ? w : m;
    }
  return m;
}
template <int K, int C>
struct LaneSpan {
  static constexpr int first() { return lane_span_first(K, C); }
  static constexpr int last() { return lane_span_last(K, C); }
  // Words fetched from neighbouring lanes, per array.
  static constexpr int neighbour_words = (last() - 3) - first();
};

// Lane-form modes whose horizontal pass takes the neighbours' words by warp
// shuffle from registers instead of through the warp's shared V row: those
// that need at most kShuffleWords neighbour words per lane array.
#ifndef KCV_SHUFFLE_WORDS
#define KCV_SHUFFLE_WORDS 6
#endif
// Whether the horizontal pass of (mode, k, c) goes through the shared V rows
// (host and device); Sobel and the shuffle modes need none.
__host__ __device__ constexpr bool uses_v_rows(int mode, int k, int c) {
  return mode == MODE_BLURDOWN ||
         (mode != MODE_SOBEL_X && mode != MODE_SOBEL_Y &&
          (mode == MODE_SEP_U16 || mode == MODE_SEP_S16
               ? 2 * (k / 2) * c > KCV_SHUFFLE_WORDS  // one 32-bit word per element
               : (lane_span_last(k, c) - 3) - lane_span_first(k, c) > KCV_SHUFFLE_WORDS));
}
template <int MODE, int K, int C>
constexpr bool shuffle_horizontal() {
  return !ModeTraits<MODE>::SOBEL && !uses_v_rows(MODE, K, C);
}

// Fills the words of lo/hi that the horizontal pass reads from the lane's
// vertical results `v` (lo words 0..3, hi words 4..7) and its neighbours'.
// Halo lanes (whose results are discarded) may receive wrapped values.
template <int MODE, int K, int C, int NW>
__device__ __forceinline__ void lanes_from_registers(const uint32_t (&v)[8], uint32_t (&lo)[NW],
                                                     uint32_t (&hi)[NW]) {
  using G = Geo<MODE, K, C>;
  constexpr int HW = G::HW;
  static_for<LaneSpan<K, C>::first(), LaneSpan<K, C>::last() + 1>([&](auto kc) {
    constexpr int k = decltype(kc)::value;
    constexpr int delta = floor_div(k, 4), word = k - 4 * delta;
    static_assert(HW + k >= 0 && HW + k < NW, "word outside the lane arrays");
    static_assert(delta >= -G::HC && delta <= G::HC, "neighbour beyond the halo lanes");
    if constexpr (delta == 0) {
      lo[HW + k] = v[word];
      hi[HW + k] = v[4 + word];
    } else if constexpr (delta < 0) {
      lo[HW + k] = __shfl_up_sync(0xffffffffu, v[word], -delta);
      hi[HW + k] = __shfl_up_sync(0xffffffffu, v[4 + word], -delta);
    } else {
      lo[HW + k] = __shfl_down_sync(0xffffffffu, v[word], delta);
      hi[HW + k] = __shfl_down_sync(0xffffffffu, v[4 + word], delta);
    }
  });
}

// The 16 output bytes of the thread for the lane-form modes.  The V row
// holds, per lane, its lo words then (128 words later) its hi words; with
// REGS the words come from `v` and the neighbours' registers instead.
template <int MODE, int K, int C, bool NARROW, bool REGS = false>
__device__ __forceinline__ uint4 horizontal_lanes(const uint32_t *vlo_s, const uint32_t *vhi_s,
                                                  int tid, const uint32_t (&v)[8], const Taps &tp) {
  using G = Geo<MODE, K, C>;
  constexpr int R = K / 2, HW = G::HW, NW = G::NW;
  uint32_t lo[NW], hi[NW];
  if constexpr (REGS) {
    lanes_from_registers<MODE, K, C, NW>(v, lo, hi);
  } else {
    const int base = 4 * tid - HW;
#pragma unroll
    for (int k = 0; k < NW; k += 4) {
      const uint4 a = *reinterpret_cast<const uint4 *>(vlo_s + base + k);
      const uint4 b = *reinterpret_cast<const uint4 *>(vhi_s + base + k);
      lo[k] = a.x; lo[k + 1] = a.y; lo[k + 2] = a.z; lo[k + 3] = a.w;
      hi[k] = b.x; hi[k + 1] = b.y; hi[k + 2] = b.z; hi[k + 3] = b.w;
    }
  }
  // Taps outer, the eight lane pairs (J = 2*I + P) inner.
  uint32_t acc[8];
  uint32_t out[4];
  if constexpr (MODE == MODE_SIGMA || (MODE == MODE_BINOM && K <= 5)) {
    // Sums stay inside 16-bit lanes: sigma weights sum to 256, binomial 5x5
    // to 256 (3x3 to 16) before the rounding shift.
    static_for<0, 8>([&](auto jc) {
      constexpr int J = decltype(jc)::value;
      uint32_t c0;
      if constexpr (MODE == MODE_SIGMA) c0 = 0x00800080u + tp.y[R] * pair_at<HW, NW, J / 2, J % 2, 0>(lo, hi);
      else c0 = (1u << (Binomial<K>::shift - 1)) * 0x00010001u +
                Binomial<K>::c(R) * pair_at<HW, NW, J / 2, J % 2, 0>(lo, hi);
      acc[J] = c0;
    });
    static_for<1, R + 1>([&](auto dc) {
      constexpr int D = decltype(dc)::value;
      static_for<0, 8>([&](auto jc) {
        constexpr int J = decltype(jc)::value;
        const uint32_t pr = pair_at<HW, NW, J / 2, J % 2, -D * C>(lo, hi) +
                            pair_at<HW, NW, J / 2, J % 2, D * C>(lo, hi);
        if constexpr (MODE == MODE_SIGMA) acc[J] += tp.y[R - D] * pr;
        else acc[J] += Binomial<K>::c(R - D) * pr;
      });
    });
    static_for<0, 4>([&](auto ic) {
      constexpr int I = decltype(ic)::value;
      if constexpr (MODE == MODE_BINOM && K == 3)
        out[I] = __byte_perm((acc[2 * I] >> 4) & 0x00FF00FFu, (acc[2 * I + 1] >> 4) & 0x00FF00FFu,
                             0x6240);
      else
        out[I] = __byte_perm(acc[2 * I], acc[2 * I + 1], 0x7351);  // high byte of each lane
    });
  } else if constexpr (MODE == MODE_SEP_U8) {
    static_for<0, 8>([&](auto jc) { acc[decltype(jc)::value] = 0; });
    static_for<0, K>([&](auto tc) {
      constexpr int T = decltype(tc)::value;
      static_for<0, 8>([&](auto jc) {
        constexpr int J = decltype(jc)::value;
        const uint32_t p = tp.x[T] * pair_at<HW, NW, J / 2, J % 2, (T - R) * C>(lo, hi);
        if constexpr (NARROW) acc[J] += p;
        else acc[J] += vmin_u16x2(p, 0x00FF00FFu);
      });
    });
    static_for<0, 4>([&](auto ic) {
      constexpr int I = decltype(ic)::value;
      out[I] = __byte_perm(vmin_u16x2(acc[2 * I], 0x00FF00FFu),
                           vmin_u16x2(acc[2 * I + 1], 0x00FF00FFu), 0x6240);
    });
  } else {
    // Binomial 7x7 / 9x9 need 32-bit sums (u32 in the reference, :220-279, :395-438).
    using B = Binomial<K>;
    static_for<0, 4>([&](auto ic) {
      constexpr int I = decltype(ic)::value;
      uint32_t res[2];
      static_for<0, 2>([&](auto pc) {
        constexpr int P = decltype(pc)::value;
        uint32_t a0 = 1u << (B::shift - 1), a1 = a0;
        static_for<0, K>([&](auto tc) {
          constexpr int T = decltype(tc)::value;
          const uint32_t pr = pair_at<HW, NW, I, P, (T - R) * C>(lo, hi);
          a0 += B::c(T) * (pr & 0xFFFFu);
          a1 += B::c(T) * (pr >> 16);
        });
        res[P] = ((a0 >> B::shift) & 0xFFu) | (((a1 >> B::shift) & 0xFFu) << 16);
      });
      out[I] = __byte_perm(res[0], res[1], 0x6240);  // low byte of each lane
    });
  }
  return make_uint4(out[0], out[1], out[2], out[3]);
}

// Sobel derivatives: the 16 s16 outputs of the thread (32 bytes, o0 = elements
// 0..7, o1 = 8..15).  Every per-lane result r in [-1020, 1020] is formed as
// 0x8000 + r inside its 16-bit lane (no carry or borrow crosses lanes), and
// flipping bit 15 turns that into r's two's-complement bits.
//   X: V[x + C] - V[x - C] of the [1 2 1] vertical sums (sobel_neon.cpp:55-60);
//   Y: V[x - C] + 2 V[x] + V[x + C] of the +256-biased [-1 0 1] vertical
//      differences (sobel_neon.cpp:111-118), bias 4 * 256 removed.
//
// A 3-tap filter over at most 4 channels reaches one 32-bit word past the
// lane's own four in each of its two lane arrays, so the neighbours' edge
// words come by warp shuffle straight from registers (`v` = lo words 0..3,
// hi words 4..7 of the lane's vertical results); lanes 0 and 31 are halo
// lanes whose results are discarded.
template <int MODE, int C>
__device__ __forceinline__ void horizontal_sobel(const uint32_t (&v)[8], uint4 &o0, uint4 &o1) {
  using G = Geo<MODE, 3, C>;
  constexpr int HW = G::HW, NW = G::NW;
  static_assert(HW == 4, "one halo chunk per side");
  uint32_t lo[NW], hi[NW];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    lo[HW + k] = v[k];
    hi[HW + k] = v[4 + k];
  }
  lo[HW - 1] = __shfl_up_sync(0xffffffffu, v[3], 1);
  hi[HW - 1] = __shfl_up_sync(0xffffffffu, v[7], 1);
  lo[HW + 4] = __shfl_down_sync(0xffffffffu, v[0], 1);
  hi[HW + 4] = __shfl_down_sync(0xffffffffu, v[4], 1);
  uint32_t acc[8];
  static_for<0, 8>([&](auto jc) {
    constexpr int J = decltype(jc)::value;
    const uint32_t l = pair_at<HW, NW, J / 2, J % 2, -C>(lo, hi);
    const uint32_t r = pair_at<HW, NW, J / 2, J % 2, C>(lo, hi);
    if constexpr (MODE == MODE_SOBEL_X) {
      acc[J] = r - l + 0x80008000u;
    } else {
      const uint32_t m = pair_at<HW, NW, J / 2, J % 2, 0>(lo, hi);
      acc[J] = l + r + 2u * m + (0x8000u - 4u * 256u) * 0x00010001u;
    }
  });
  // acc[2I] holds elements (4I, 4I + 2), acc[2I + 1] elements (4I + 1, 4I + 3).
  uint32_t w[8];
  static_for<0, 4>([&](auto ic) {
    constexpr int I = decltype(ic)::value;
    w[2 * I] = __byte_perm(acc[2 * I], acc[2 * I + 1], 0x5410) ^ 0x80008000u;
    w[2 * I + 1] = __byte_perm(acc[2 * I], acc[2 * I + 1], 0x7632) ^ 0x80008000u;
  });
  o0 = make_uint4(w[0], w[1], w[2], w[3]);
  o1 = make_uint4(w[4], w[5], w[6], w[7]);
}

// u16 / s16 separable: the V row holds 8 32-bit elements per lane (u16
// values clamped to 65535, or s16 vertical sums), lane-major.
template <int MODE, int K, int C, bool NARROW, bool REGS = false>
__device__ __forceinline__ uint4 horizontal_wide(const uint32_t *v_s, int tid,
                                                 const uint32_t (&own)[8], const Taps &tp) {
  using G = Geo<MODE, K, C>;
  constexpr int R = K / 2, HE = 2 * G::HW, NE = 8 + 2 * HE;  // elements
  uint32_t v[NE];
  if constexpr (REGS) {
    // Elements -R*C .. 7+R*C around the lane's own eight: the neighbours'
    // come by shuffle (halo lanes, whose results are discarded, may wrap).
    static_for<-R * C, 8 + R * C>([&](auto ec) {
      constexpr int e = decltype(ec)::value;
      constexpr int delta = floor_div(e, 8), idx = e - 8 * delta;
      static_assert(delta >= -G::HC && delta <= G::HC, "neighbour beyond the halo lanes");
      if constexpr (delta == 0) v[HE + e] = own[idx];
      else if constexpr (delta < 0) v[HE + e] = __shfl_up_sync(0xffffffffu, own[idx], -delta);
      else v[HE + e] = __shfl_down_sync(0xffffffffu, own[idx], delta);
    });
  } else {
    const int base = 8 * tid - HE;
#pragma unroll
    for (int k = 0; k < NE; k += 4) {
      const uint4 a = *reinterpret_cast<const uint4 *>(v_s + base + k);
      v[k] = a.x; v[k + 1] = a.y; v[k + 2] = a.z; v[k + 3] = a.w;
    }
  }
  uint32_t o[8];
  if constexpr (MODE == MODE_SEP_U16) {
    uint32_t acc[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) acc[e] = 0;
    static_for<0, K>([&](auto tc) {
      constexpr int T = decltype(tc)::value;
#pragma unroll
      for (int e = 0; e < 8; ++e) {
        const uint32_t p = tp.x[T] * v[HE + e + (T - R) * C];
        acc[e] += NARROW ? p : min(p, 0xFFFFu);
      }
    });
#pragma unroll
    for (int e = 0; e < 8; ++e) o[e] = min(acc[e], 0xFFFFu);
  } else if constexpr (NARROW) {
    // |sum| < 2^31: plain 32-bit accumulation, then saturation to s16.
    int32_t acc[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) acc[e] = 0;
    static_for<0, K>([&](auto tc) {
      constexpr int T = decltype(tc)::value;
#pragma unroll
      for (int e = 0; e < 8; ++e)
        acc[e] += static_cast<int32_t>(tp.x[T]) * static_cast<int32_t>(v[HE + e + (T - R) * C]);
    });
#pragma unroll
    for (int e = 0; e < 8; ++e)
      o[e] = static_cast<uint32_t>(max(-32768, min(acc[e], 32767))) & 0xFFFFu;
  } else {
    // s16 extension: 64-bit horizontal accumulation, saturation to s16.
    int64_t acc[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) acc[e] = 0;
    static_for<0, K>([&](auto tc) {
      constexpr int T = decltype(tc)::value;
#pragma unroll
      for (int e = 0; e < 8; ++e)
        acc[e] += static_cast<int64_t>(static_cast<int32_t>(tp.x[T])) *
                  static_cast<int32_t>(v[HE + e + (T - R) * C]);
    });
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      const int64_t c = acc[e] > 32767 ? 32767 : (acc[e] < -32768 ? -32768 : acc[e]);
      o[e] = static_cast<uint32_t>(c) & 0xFFFFu;
    }
  }
  return make_uint4(o[0] | (o[1] << 16), o[2] | (o[3] << 16), o[4] | (o[5] << 16),
                    o[6] | (o[7] << 16));
}

// blur_and_downsample: the thread produces the 8 destination bytes whose
// source centres lie in its chunk.  Destination element o (absolute) has
// channel ch = o % C and source centre 2*o - ch; taps are centre + d*C with
// the binomial [1 4 6 4 1] (blur_and_downsample_neon.cpp:128-177).
template <int C>
__device__ __forceinline__ uint2 horizontal_blurdown(const uint32_t *vlo_s, const uint32_t *vhi_s,
                                                     long out_elem0, int span_elem0) {
  uint32_t o[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const long oe = out_elem0 + k;
    const int ch = static_cast<int>(oe % C);
    const int centre = static_cast<int>(2 * oe - ch - span_elem0);  // index into the span
    uint32_t acc = 128;
#pragma unroll
    for (int d = -2; d <= 2; ++d) {
      const int e = centre + d * C;
      const uint32_t *arr = (e & 1) ? vhi_s : vlo_s;
      const uint32_t word = arr[e >> 2];
      const uint32_t val = ((e >> 1) & 1) ? (word >> 16) : (word & 0xFFFFu);
      const uint32_t c = (d == 0) ? 6u : ((d == 1 || d == -1) ? 4u : 1u);
      acc += c * val;
    }
    o[k] = (acc >> 8) & 0xFFu;
  }
  return make_uint2(o[0] | (o[1] << 8) | (o[2] << 16) | (o[3] << 24),
                    o[4] | (o[5] << 8) | (o[6] << 16) | (o[7] << 24));
}

// ---------------------------------------------------------------------------
// CTA organisation.  Each warp owns 32 consecutive chunks (16 bytes of a row
// per lane): an interior of 32 - 2*HC chunks plus HC halo chunks on either
// side, which overlap the neighbouring warps' interiors.  A warp therefore
// needs no other warp's data and synchronises only with __syncwarp; the warps
// of a CTA share the TMA ring through full/empty mbarrier pairs, and lane 0 of
// one warp issues the copies between its own blocks of rows.
struct CtaShape {
  int warps;        // warps of the CTA
  int wi;           // interior chunks per warp
  int span_chunks;  // chunks of a row the CTA reads: warps * wi + 2 * HC
  int boxes;        // span boxes per row
  int span_bytes;   // boxes * box width
};

__host__ __device__ inline CtaShape cta_shape(int threads, int hc, int lbw) {
  CtaShape s;
  const int bw = 1 << lbw;
  s.warps = threads / 32;
  s.wi = 32 - 2 * hc;
  s.span_chunks = s.warps * s.wi + 2 * hc;
  s.boxes = (s.span_chunks * kChunk + bw - 1) / bw;
  s.span_bytes = s.boxes * bw;
  return s;
}

// Chunks per warp that can hang over the image's left/right edge and are
// rebuilt in a per-warp edge area: at most HC on the left plus HC + 1 on the
// right.
__host__ __device__ constexpr int edge_slots(int hc) { return 2 * hc + 1; }

constexpr uint32_t kBarBytes = 256;      // full[stages] + empty[stages], stages <= 16
constexpr uint32_t kVRowBytes = 32 * 32;  // one V row of a warp: 32 lanes x 8 words

// Shared memory of one CTA:
//   [0, 256)     mbarriers full[stages], empty[stages] (stages <= 16)
//   ring         TMA: [box][ring row][box bytes]; plain loads: [ring row][warp][lane][16 B]
//   wrap         (TMA with a WRAP border) [2][ring row][256 B]
//   edge         (TMA) per warp [ring row][edge_slots][16 B]: chunks rebuilt by
//                generic stores (never written by TMA, so no proxy fence)
//   V            per warp [2][kVRowBytes] (double-buffered vertical row)
struct SmemLayout {
  uint32_t ring_off, ring_rows, wrap_off, edge_off, edge_warp_bytes, v_off, total;
};

__host__ __device__ inline SmemLayout smem_layout(int mode, int k, int c, int threads, int hc,
                                                  int lbw, int stage_rows, int stages,
                                                  bool use_tma, bool wrap) {
  const CtaShape s = cta_shape(threads, hc, lbw);
  SmemLayout l;
  l.ring_rows = static_cast<uint32_t>(stage_rows * stages);
  l.ring_off = kBarBytes;
  const uint32_t ring_bytes = use_tma ? l.ring_rows * static_cast<uint32_t>(s.span_bytes)
                                      : l.ring_rows * s.warps * 32 * kChunk;
  l.wrap_off = l.ring_off + ring_bytes;
  const uint32_t wrap_bytes = (use_tma && wrap) ? 2 * l.ring_rows * 256 : 0;
  l.edge_off = l.wrap_off + wrap_bytes;
  l.edge_warp_bytes = use_tma ? l.ring_rows * edge_slots(hc) * kChunk : 0;
  l.v_off = l.edge_off + s.warps * l.edge_warp_bytes;
  l.total = l.v_off + (uses_v_rows(mode, k, c) ? s.warps * 2 * kVRowBytes : 0u);
  return l;
}

constexpr uint64_t kWaitLimitNs = 2000000000ull;  // 2 s for any device-side wait

// The tensor maps of one job.  Span maps view the row in units of 1 << (lbw-8)
// bytes (1 or 8) so that one box is 256 such units wide; wrap maps always use
// bytes.
struct TmaMaps {
  const CUtensorMap *span, *span_row, *wrap, *wrap_row;
};

// ---------------------------------------------------------------------------
// One tile: strip `strip` x band `band` of job `j`.  `gstage` counts ring
// stages used by this CTA so far (mbarrier phases continue across tiles).
// stage_rows and stages are powers of two.  SHIFT_STORES compiles the
// aligned-block stores for destination rows that are not 16-byte aligned
// (store_shifted); without it such rows are written byte by byte.
template <int MODE, int K, int C, bool NARROW, bool SHIFT_STORES>
__device__ __forceinline__ void run_tile(const FilterJob &j, const TmaMaps &maps, int strip,
                                         int band, uint8_t *smem, uint32_t &gstage,
                                         int *err_flag, bool &timed_out) {
  using G = Geo<MODE, K, C>;
  constexpr int ES = G::ES;
  constexpr int HC = G::HC;
  constexpr int E = kChunk / ES;
  constexpr int M = block_out_rows(MODE, K);

  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int lbw = j.box_lbw;
  const CtaShape sh = cta_shape(blockDim.x, HC, lbw);
  const int rb = j.stage_rows, ns = j.stages;
  const int lrb = __ffs(rb) - 1;
  const bool use_tma = j.use_tma != 0;
  const SmemLayout L = smem_layout(MODE, K, C, blockDim.x, HC, lbw, rb, ns, use_tma,
                                   j.border == BORDER_WRAP);
  uint64_t *full = reinterpret_cast<uint64_t *>(smem);
  uint64_t *empty = full + ns;
  uint8_t *const ring = smem + L.ring_off;
  uint8_t *const wrap = smem + L.wrap_off;
  const int ring_rows = static_cast<int>(L.ring_rows);
  // Ring position of the tile's first stage: slot (gstage mod stages) and
  // use count (gstage / stages, whose parity is the mbarrier phase).
  const int base_slot = static_cast<int>(gstage % static_cast<uint32_t>(ns));
  const uint32_t base_use = gstage / static_cast<uint32_t>(ns);
  struct RingPos {
    int slot;
    uint32_t use;
  };
  auto advance = [&](RingPos &p) {
    if (++p.slot == ns) {
      p.slot = 0;
      ++p.use;
    }
  };

  const int oy0 = band * j.tile_rows + M * min(band, j.big_bands);
  const int orows = band == j.row_tiles - 1 ? j.out_height - oy0
                                            : j.tile_rows + (band < j.big_bands ? M : 0);
  const int iy0 = MODE == MODE_BLURDOWN ? 2 * oy0 - 2 : oy0 - G::R;
  const int in_rows = MODE == MODE_BLURDOWN ? 2 * orows + 3 : orows + K - 1;
  const long xs = static_cast<long>(strip) * sh.warps * sh.wi * kChunk - HC * kChunk;
  const long wc = static_cast<long>(j.width) * C;
  const long wcb = wc * ES;
  const int nstages = (in_rows + rb - 1) >> lrb;
  // The producer is lane 0 of a warp whose chunks never hang over a strip's
  // left edge (warp 1 when the CTA has three or more warps): edge warps
  // already carry the cooperative border patching.
  const int pw = sh.warps >= 3 ? 1 : 0;

  RingGeo rg;
  rg.xs = xs;
  rg.span_end = xs + sh.span_bytes;
  rg.wcb = wcb;
  rg.lbw = lbw;
  rg.ring_rows = ring_rows;
  {
    // The wrap areas are filled only for a WRAP border on a strip that touches
    // exactly one side of the image (a strip spanning both sides already
    // holds the far end of the row).
    const bool left = xs < 0, right = rg.span_end > wcb;
    rg.wrap_left = use_tma && j.border == BORDER_WRAP && left && !right;
    rg.wrap_right = use_tma && j.border == BORDER_WRAP && right && !left;
    const long hb = static_cast<long>(G::HALO_ELEMS) * ES;
    rg.wrapl_x = wcb - hb > 0 ? ((wcb - hb) & ~15L) : 0;
  }

  // ======================= producer (lane 0 of warp pw) ======================
  // fn(map, x in map units, destination, box width) for every box of the
  // rows starting at ring row `rr`.
  const int bw = 1 << lbw, unit_shift = lbw - 8;  // span map unit = 1 << unit_shift bytes
  auto for_each_box = [&](int rr, bool single_row, auto &&fn) {
    for (int b = 0; b < sh.boxes; ++b) {
      const long x = xs + static_cast<long>(b) * bw;
      if (x < wcb && x + bw > 0)
        fn(single_row ? maps.span_row : maps.span, x >> unit_shift,
           ring + (b * ring_rows + rr) * bw, static_cast<uint32_t>(bw));
    }
    if (rg.wrap_left) fn(single_row ? maps.wrap_row : maps.wrap, rg.wrapl_x, wrap + rr * 256, 256u);
    if (rg.wrap_right)
      fn(single_row ? maps.wrap_row : maps.wrap, 0L, wrap + (ring_rows + rr) * 256, 256u);
  };
  // Copies stage s into its slot (the slot must be free).  Rows inside the
  // image arrive as stage_rows-high boxes; a stage that reaches outside gets
  // one single-row box per row of its border-mapped source row instead (none
  // for a CONSTANT border).
  auto issue_stage = [&](int s, int slot) {
    uint64_t *bar = &full[slot];
    const int y = iy0 + s * rb;
    const int rr0 = slot * rb;
    const bool rows_in = y >= 0 && y + rb <= j.height;
    uint32_t tx = 0;
    if (rows_in) {
      for_each_box(rr0, false, [&](const CUtensorMap *, long, uint8_t *, uint32_t w) { tx += w * rb; });
    } else {
      for (int r = 0; r < rb; ++r)
        if (map_index(y + r, j.height, j.border) >= 0)
          for_each_box(rr0 + r, true, [&](const CUtensorMap *, long, uint8_t *, uint32_t w) { tx += w; });
    }
    if (tx == 0) {
      mbar_arrive(bar);
      return;
    }
    mbar_arrive_expect_tx(bar, tx);
    if (rows_in) {
      for_each_box(rr0, false, [&](const CUtensorMap *m, long x, uint8_t *d, uint32_t) {
        tma_load_2d(d, m, static_cast<int>(x), y, bar);
      });
    } else {
      for (int r = 0; r < rb; ++r) {
        const int my = map_index(y + r, j.height, j.border);
        if (my >= 0)
          for_each_box(rr0 + r, true, [&](const CUtensorMap *m, long x, uint8_t *d, uint32_t) {
            tma_load_2d(d, m, static_cast<int>(x), my, bar);
          });
      }
    }
  };
  // Called by warp pw between its blocks: issues every stage up to
  // `last_needed` (waiting, with a time limit, for its slot to be released),
  // then as many further stages as have free slots.
  int issued = 0;
  RingPos ppos{base_slot, base_use};
  auto produce = [&](int last_needed) {
    if (use_tma && lane == 0) {
      while (issued < nstages && !timed_out) {
        const int slot = ppos.slot;
        const uint32_t use = ppos.use;
        if (use > 0) {
          if (issued <= last_needed) {
            if (!mbar_wait_bounded(&empty[slot], (use - 1) & 1u, kWaitLimitNs)) {
              timed_out = true;
              atomicOr(err_flag, 1);
              break;
            }
          } else if (!mbar_test_wait(&empty[slot], (use - 1) & 1u)) {
            break;
          }
        }
        issue_stage(issued, slot);
        ++issued;
        advance(ppos);
      }
    }
    __syncwarp();
  };

  // ======================= consumers (every warp) =======================
  const int cidx = warp * sh.wi + lane;  // chunk index within the CTA span
  const long xb = xs + static_cast<long>(cidx) * kChunk;
  const bool chunk_in = xb >= 0 && xb + kChunk <= wcb;
  // Chunks that start past the right halo only feed discarded lanes.
  const bool active = xb < wcb + HC * kChunk;
  const bool emits = lane >= HC && lane < 32 - HC;
  // Destination rows all start 16-byte aligned when base and stride are.
  const bool dst_rows_aligned =
      ((reinterpret_cast<uintptr_t>(j.dst) | static_cast<uintptr_t>(j.dst_stride)) & 15) == 0;
  // Sobel chunks are 32 destination bytes: one 32-byte store when rows allow.
  const bool dst_rows_aligned32 =
      ((reinterpret_cast<uintptr_t>(j.dst) | static_cast<uintptr_t>(j.dst_stride)) & 31) == 0;
  // This lane writes a whole 16-byte chunk with one vector store.
  const bool stores = emits && active && xb < wcb;
  const bool full_store = stores && dst_rows_aligned && xb >= 0 && xb + kChunk <= wcb;
  // Destination rows that are not 16-byte aligned: a lane whose chunk lies
  // inside the row writes the aligned 16-byte block that ends inside its
  // chunk, assembled from its own result and the previous lane's; the first
  // and last such lanes of the warp also write the bytes of their chunk that
  // no block covers (the modes with 16 destination bytes per chunk).
  const bool shift_store = SHIFT_STORES && !ModeTraits<MODE>::SOBEL && MODE != MODE_BLURDOWN && stores &&
                           !dst_rows_aligned && xb >= 0 && xb + kChunk <= wcb;
  const unsigned shift_mask = SHIFT_STORES ? __ballot_sync(0xffffffffu, shift_store) : 0u;
  const bool shift_first = shift_store && !((shift_mask >> (lane - 1)) & 1u);
  const bool shift_last = shift_store && !((shift_mask >> (lane + 1)) & 1u);
  const uint32_t bv_elem = ES == 1 ? (static_cast<uint32_t>(j.border_value) & 0xFFu)
                                   : (static_cast<uint32_t>(j.border_value) & 0xFFFFu);
  const uint32_t bv_word = ES == 1 ? bv_elem * 0x01010101u : bv_elem * 0x00010001u;
  // Without TMA every lane owns a 16-byte slot per ring row.
  const int own_pitch = sh.warps * 32 * kChunk;
  auto own_slot = [&](int l) { return ring + (warp * 32 + l) * kChunk; };
  // Lanes whose chunk is not plain image data in every row: hanging over the
  // left/right edge, or (without TMA) not loadable with 16-byte loads.
  // (load_chunk_fast succeeds in every row when the chunk is 16-byte aligned
  // in every row, or when the two aligned blocks around it stay in the row
  // whatever the row's misalignment.)
  bool self_load_ok = chunk_in;
  if (!use_tma && chunk_in) {
    const uintptr_t pa = reinterpret_cast<uintptr_t>(j.src) + static_cast<uintptr_t>(xb);
    self_load_ok = ((pa | static_cast<uintptr_t>(j.src_stride)) & 15) == 0 ||
                   (xb >= 16 && xb + 32 <= wcb);
  }
  const unsigned coop_lanes = __ballot_sync(0xffffffffu, active && !self_load_ok);
  // With TMA, chunks rebuilt by the warp live in the edge area at compact slot
  // `edge_slot`; every other chunk is read where TMA put it.
  uint8_t *const edge_warp = smem + L.edge_off + warp * L.edge_warp_bytes;
  const int edge_pitch = edge_slots(HC) * kChunk;
  const int edge_slot = __popc(coop_lanes & ((1u << lane) - 1u));
  const bool from_edge = use_tma && ((coop_lanes >> lane) & 1u);
  const uint8_t *lane_base;
  uint32_t lane_pitch;
  if (!use_tma) {
    lane_base = own_slot(lane);
    lane_pitch = static_cast<uint32_t>(own_pitch);
  } else if (from_edge) {
    lane_base = edge_warp + edge_slot * kChunk;
    lane_pitch = static_cast<uint32_t>(edge_pitch);
  } else {
    const int o = cidx * kChunk;  // offset within the span
    lane_base = ring + (o >> lbw) * ring_rows * bw + (o & (bw - 1));
    lane_pitch = static_cast<uint32_t>(bw);
  }

  Taps tp;
  if constexpr (MODE == MODE_SIGMA) {
#pragma unroll
    for (int t = 0; t <= K / 2; ++t) tp.y[t] = static_cast<uint32_t>(j.wy[t]);
  } else if constexpr (MODE != MODE_BINOM && MODE != MODE_BLURDOWN && !ModeTraits<MODE>::SOBEL) {
#pragma unroll
    for (int t = 0; t < K; ++t) {
      tp.y[t] = static_cast<uint32_t>(j.wy[t]);
      tp.x[t] = static_cast<uint32_t>(j.wx[t]);
    }
  }

  // Readies stage s for this warp.  With TMA: waits for the copies.  Without:
  // every lane loads its own chunk of each row.  Rows lying in a CONSTANT
  // border get the border value in every chunk.  Then the warp jointly fills
  // the chunks in `coop_lanes`, one (row, element) pair per lane: border-mapped
  // elements come from the staged row (or, without TMA, every element from
  // global memory).  Lanes that share a chunk with a neighbouring warp write
  // identical bytes.
  RingPos rpos{base_slot, base_use}, lpos{base_slot, base_use};
  auto prepare_stage = [&](int s) {
    const int slot = rpos.slot;
    const uint32_t phase = rpos.use & 1u;
    advance(rpos);
    if (use_tma && !timed_out && !mbar_wait_bounded(&full[slot], phase, kWaitLimitNs)) {
      timed_out = true;
      atomicOr(err_flag, 1);
    }
    // Interior warps of an interior stage: the copies are all there is.
    if (use_tma && coop_lanes == 0u && j.border != BORDER_CONSTANT) return;
    const int rows = min(rb, in_rows - s * rb);
    if (!use_tma) {
#pragma unroll 1
      for (int r = 0; r < rows; ++r) {
        const int iy = iy0 + s * rb + r;
        uint4 *dst = reinterpret_cast<uint4 *>(own_slot(lane) + (slot * rb + r) * own_pitch);
        if (j.border == BORDER_CONSTANT && (iy < 0 || iy >= j.height)) {
          if (active) *dst = make_uint4(bv_word, bv_word, bv_word, bv_word);
        } else if (active && self_load_ok) {
          uint4 v;
          load_chunk_fast(j.src + static_cast<int64_t>(map_index(iy, j.height, j.border)) *
                                      j.src_stride,
                          xb, wcb, v);
          *dst = v;
        }
      }
    }
    // TMA never fetches rows of a CONSTANT border: every lane fills its own
    // chunk of them (lanes sharing a chunk write the same bytes), and fences
    // those generic writes against the TMA copy that will reuse the slot.
    if (use_tma && j.border == BORDER_CONSTANT) {
      const int y0 = iy0 + s * rb;
      if (y0 < 0 || y0 + rows > j.height) {
        for (int r = 0; r < rows; ++r)
          if (y0 + r < 0 || y0 + r >= j.height)
            *reinterpret_cast<uint4 *>(const_cast<uint8_t *>(lane_base) + (slot * rb + r) * lane_pitch) =
                make_uint4(bv_word, bv_word, bv_word, bv_word);
        fence_proxy_async_smem();
      }
    }
    int k = 0;
    for (unsigned m = coop_lanes; m; m &= m - 1, ++k) {
      const int l = __ffs(m) - 1;
      const int x0 = static_cast<int>((xs + static_cast<long>(warp * sh.wi + l) * kChunk) / ES);
      uint8_t *lbase = use_tma ? edge_warp + k * kChunk : own_slot(l);
      const int lpitch = use_tma ? edge_pitch : own_pitch;
#pragma unroll 1
      for (int idx = lane; idx < rows * E; idx += 32) {
        const int r = idx / E, e = idx % E;
        const int iy = iy0 + s * rb + r;
        if (j.border == BORDER_CONSTANT && (iy < 0 || iy >= j.height)) continue;
        const int rr = slot * rb + r;
        const int x = x0 + e;
        const bool inside = x >= 0 && x < static_cast<int>(wc);
        int me = x;
        if (!inside) {
          const int col = x >= 0 ? x / C : -((-x + C - 1) / C);
          const int mc = map_index(col, j.width, j.border);
          me = mc < 0 ? -1 : mc * C + (x - col * C);
        }
        uint32_t v;
        if (me < 0) {
          v = bv_elem;
        } else if (use_tma) {
          v = staged_byte(ring, wrap, rg, rr, static_cast<long>(me) * ES);
          if (ES == 2) v |= staged_byte(ring, wrap, rg, rr, static_cast<long>(me) * ES + 1) << 8;
        } else {
          const uint8_t *grow =
              j.src + static_cast<int64_t>(map_index(iy, j.height, j.border)) * j.src_stride;
          v = ES == 1 ? __ldg(grow + me) : __ldg(reinterpret_cast<const uint16_t *>(grow) + me);
        }
        uint8_t *dst = lbase + rr * lpitch + e * ES;
        dst[0] = static_cast<uint8_t>(v);
        if (ES == 2) dst[1] = static_cast<uint8_t>(v >> 8);
      }
    }
    __syncwarp();
  };
  // Hands stage s back to the producer once every lane of the warp has read it.
  auto release_stage = [&]() {
    if (!use_tma) return;
    const int slot = lpos.slot;
    advance(lpos);
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[slot]);
  };

  uint32_t *const vwarp = reinterpret_cast<uint32_t *>(smem + L.v_off + warp * 2 * kVRowBytes);
  uint8_t *const dst_base = j.dst;
  const int64_t dst_stride = j.dst_stride;
  // Lanes outside the interior compute a duplicate of their nearest interior
  // neighbour's horizontal pass (never stored), so that no branch is needed.
  const int hlane = min(max(lane, HC), 31 - HC);
  const bool partial_store = stores && !full_store && !shift_store;
  constexpr int NIN = block_in_rows(MODE, K);

  // ---- output rows in blocks of M.  Before a block, the stages holding only
  // rows below the block are released FIRST, then the stages the block reads
  // are readied.  A block reads at most floor((stage_rows - 1 + NIN - 1) /
  // stage_rows) + 1 stages; with at least that many stages in the ring, the
  // slot of every stage a warp waits for was released by all warps (each has
  // released everything below its own block), so the producer can always
  // issue what the most advanced warp waits for.
  int ready = 0, released = 0;
  int rq = base_slot * rb;  // ring row of the block's first source row
  for (int ob = 0; ob < orows; ob += M) {
    const int q0 = MODE == MODE_BLURDOWN ? 2 * ob : ob;
    const int last_stage = (min(q0 + NIN, in_rows) - 1) >> lrb;
    for (; released < ready && ((released + 1) << lrb) <= q0; ++released) release_stage();
    if (warp == pw) produce(last_stage);
    for (; ready <= last_stage; ++ready) prepare_stage(ready);
    // Rows past the band's end (last block) read stale ring rows; they only
    // feed output rows that are not stored.
    uint32_t v[M][8];
    vertical_block<MODE, K, NARROW>(lane_base, lane_pitch, static_cast<uint32_t>(rq),
                                    static_cast<uint32_t>(ring_rows), tp, v);
    rq += MODE == MODE_BLURDOWN ? 2 * M : M;
    if (rq >= ring_rows) rq -= ring_rows;
    // ---- horizontal pass + store, one output row at a time.  Shuffle modes
    // (and Sobel) take the neighbours' words from registers.  The others go
    // through the warp's two V rows: write row m, __syncwarp, read it; row
    // m + 2 reuses the buffer only after the __syncwarp of row m + 1, when
    // every lane has finished reading row m.
    const int mcount = min(M, orows - ob);
    // This lane's destination chunk in the block's first row.
    uint8_t *const dblock =
        dst_base + static_cast<int64_t>(oy0 + ob) * dst_stride + xb * ModeTraits<MODE>::OSCALE;
    static_for<0, M>([&](auto mc) {
      constexpr int Mi = decltype(mc)::value;
      uint32_t *vb = vwarp + (Mi & 1) * (kVRowBytes / 4);
      constexpr bool kRegs = shuffle_horizontal<MODE, K, C>();
      if constexpr (ModeTraits<MODE>::SOBEL || kRegs) {
        // No V row: the neighbours' words come by shuffle.
      } else if constexpr (ModeTraits<MODE>::LANES) {
        *reinterpret_cast<uint4 *>(vb + 4 * lane) = make_uint4(v[Mi][0], v[Mi][1], v[Mi][2], v[Mi][3]);
        *reinterpret_cast<uint4 *>(vb + 128 + 4 * lane) =
            make_uint4(v[Mi][4], v[Mi][5], v[Mi][6], v[Mi][7]);
      } else {
        *reinterpret_cast<uint4 *>(vb + 8 * lane) = make_uint4(v[Mi][0], v[Mi][1], v[Mi][2], v[Mi][3]);
        *reinterpret_cast<uint4 *>(vb + 8 * lane + 4) =
            make_uint4(v[Mi][4], v[Mi][5], v[Mi][6], v[Mi][7]);
      }
      if constexpr (!ModeTraits<MODE>::SOBEL && !kRegs) __syncwarp();
      if constexpr (MODE == MODE_BLURDOWN) {
        uint8_t *drow = dst_base + static_cast<int64_t>(oy0 + ob + Mi) * dst_stride;
        if (Mi < mcount) {
          if (emits && active) {
            const long ob8 = xb / 2;  // destination byte (= element) offset
            const long owc = static_cast<long>(j.out_width) * C;
            if (ob8 < owc) {
              const uint2 r = horizontal_blurdown<C>(vb, vb + 128, ob8,
                                                     static_cast<int>(xb - lane * kChunk));
              if (ob8 + 8 <= owc && (reinterpret_cast<uintptr_t>(drow + ob8) & 7) == 0) {
                *reinterpret_cast<uint2 *>(drow + ob8) = r;
              } else {
                const uint32_t w2[2] = {r.x, r.y};
                for (int k = 0; k < 8 && ob8 + k < owc; ++k)
                  drow[ob8 + k] = static_cast<uint8_t>(w2[k >> 2] >> (8 * (k & 3)));
              }
            }
          }
        }
      } else if constexpr (ModeTraits<MODE>::SOBEL) {
        // 32 destination bytes per chunk (s16 per source byte).
        uint4 r0, r1;
        horizontal_sobel<MODE, C>(v[Mi], r0, r1);
        uint8_t *drow = dblock + Mi * dst_stride;
        const bool row_ok = Mi < mcount;
        if (full_store && row_ok) {
          if (dst_rows_aligned32) {
            st_v8(drow, r0, r1);
          } else {
            *reinterpret_cast<uint4 *>(drow) = r0;
            *reinterpret_cast<uint4 *>(drow + 16) = r1;
          }
        }
        if (partial_store && row_ok) {
          const uint32_t w8[8] = {r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w};
          for (int k = 0; k < kChunk && xb + k < wcb; ++k) {
            const uint32_t e = w8[k >> 1] >> (16 * (k & 1));
            drow[2 * k] = static_cast<uint8_t>(e);
            drow[2 * k + 1] = static_cast<uint8_t>(e >> 8);
          }
        }
      } else {
        // Every row of the block is computed; rows past a partial last block
        // of the band are not stored.
        uint4 r;
        if constexpr (ModeTraits<MODE>::LANES)
          r = horizontal_lanes<MODE, K, C, NARROW, kRegs>(vb, vb + 128, hlane, v[Mi], tp);
        else
          r = horizontal_wide<MODE, K, C, NARROW, kRegs>(vb, hlane, v[Mi], tp);
        uint8_t *drow = dblock + Mi * dst_stride;
        const bool row_ok = Mi < mcount;
        if (full_store && row_ok) *reinterpret_cast<uint4 *>(drow) = r;
        if (SHIFT_STORES && shift_mask != 0u) {
          // The previous lane's result ends where this lane's chunk begins.
          const uint4 pr = make_uint4(__shfl_up_sync(0xffffffffu, r.x, 1), __shfl_up_sync(0xffffffffu, r.y, 1),
                                      __shfl_up_sync(0xffffffffu, r.z, 1), __shfl_up_sync(0xffffffffu, r.w, 1));
          if (shift_store && row_ok) store_shifted(drow, pr, r, shift_first, shift_last);
        }
        if (partial_store && row_ok) {
          const uint32_t w4[4] = {r.x, r.y, r.z, r.w};
          for (int k = 0; k < kChunk && xb + k < wcb; ++k)
            drow[k] = static_cast<uint8_t>(w4[k >> 2] >> (8 * (k & 3)));
        }
      }
    });
  }
  for (; released < nstages; ++released) release_stage();
  if (use_tma && timed_out && warp == pw && lane == 0) {
    // Give copies already issued a bounded time to land before the CTA's
    // shared memory can be reused.
    RingPos d{base_slot, base_use};
    for (int s2 = 0; s2 < issued; ++s2, advance(d)) mbar_wait_bounded(&full[d.slot], d.use & 1u, kWaitLimitNs);
  }
  gstage += nstages;
}

// ---------------------------------------------------------------------------
// Launch: a grid of up to (resident CTAs per SM x SMs) CTAs that walk the
// job's tiles (strip, band) in row-major band order; threads = 32 * warps.
// Register budget: 4 resident CTAs per SM (2 for the 15/21 sizes).  Cutting
// it for 5 (96 registers, which the shuffle modes fit without spilling) was
// measured 7-11 % slower on 3840x2160 calls.
template <int MODE, int K, int C, bool NARROW>
__global__ void __launch_bounds__(128, (K >= 15 ? 2 : 4))
    sepfused_kernel(const __grid_constant__ FilterJob job, int *err_flag) {
  extern __shared__ __align__(128) uint8_t smem[];
  // The next call on the stream may start its CTAs as ours finish (they only
  // fit where ours left room); everything it reads waits for our completion.
  launch_dependents();
  if (job.use_tma) {
    if (threadIdx.x == 0) {
      prefetch_tensormap(&job.tmap);
      prefetch_tensormap(&job.tmap_row);
      uint64_t *full = reinterpret_cast<uint64_t *>(smem);
      const int warps = blockDim.x / 32;
      for (int s = 0; s < job.stages; ++s) {
        mbar_init(&full[s], 1);
        mbar_init(&full[job.stages + s], warps);
      }
      fence_mbar_init();
    }
    __syncthreads();
  }
  uint32_t gstage = 0;
  bool timed_out = false;
  const TmaMaps maps{&job.tmap, &job.tmap_row, &job.tmap_wrap, &job.tmap_wrap_row};
  const int tiles = job.strips * job.row_tiles;
  // The source may be the previous call's output: wait for that grid (set-up
  // above overlapped its tail).
  grid_dependency_wait();
  for (int t = blockIdx.x; t < tiles; t += gridDim.x)
    run_tile<MODE, K, C, NARROW, true>(job, maps, t % job.strips, t / job.strips, smem, gstage,
                                 err_flag, timed_out);
}

}  // namespace kcv
