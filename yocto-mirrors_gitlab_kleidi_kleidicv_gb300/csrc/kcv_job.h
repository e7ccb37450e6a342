// Host/device shared description of one filter job (one image, one op).
#pragma once

#include <cuda.h>
#include <stdint.h>

namespace kcv {

// What the fused stencil computes; selects the arithmetic of both passes.
enum Mode : int32_t {
  MODE_BINOM = 0,       // gaussian_blur_u8, sigma == 0 and size <= 9: u16-exact
  MODE_SIGMA = 1,       // gaussian_blur_u8 with generated weights summing to 256
  MODE_SIGMA_SAFE = 2,  // generated weights not summing to 256 (per-element path)
  MODE_SEP_U8 = 3,      // separable_filter_2d_u8, 5x5, saturating
  MODE_SEP_U16 = 4,     // separable_filter_2d_u16, 5x5, saturating
  MODE_SEP_S16 = 5,     // separable_filter_2d_s16 (extension)
  MODE_BLURDOWN = 6,    // blur_and_downsample_u8
  MODE_SOBEL_X = 7,     // sobel_3x3_horizontal_s16_u8: [1 2 1]^T x [-1 0 1]
  MODE_SOBEL_Y = 8,     // sobel_3x3_vertical_s16_u8: [-1 0 1]^T x [1 2 1]
};

// Border codes: the kleidicv_border_type_t values.
enum Border : int32_t {
  BORDER_CONSTANT = 0,
  BORDER_REPLICATE = 1,
  BORDER_REFLECT = 2,
  BORDER_WRAP = 3,
  BORDER_REVERSE = 4,
};

constexpr int kMaxTaps = 21;  // largest fused kernel size
constexpr int kChunk = 16;    // bytes of one row owned by one thread

#ifdef __CUDACC__
#define KCV_HD __host__ __device__
#else
#define KCV_HD
#endif

// The fused kernel produces output rows in blocks: block_out_rows(mode, k)
// destination rows from block_in_rows(mode, k) consecutive source rows.
KCV_HD constexpr int block_out_rows(int mode, int k) {
  return mode == MODE_BLURDOWN ? 2 : (k >= 15 ? 2 : 4);
}
KCV_HD constexpr int block_in_rows(int mode, int k) {
  return mode == MODE_BLURDOWN ? 2 * block_out_rows(mode, k) + 3 : block_out_rows(mode, k) + k - 1;
}

struct FilterJob {
  // TMA views of src (valid when use_tma).  The span maps count the row in
  // units of 1 << (box_lbw - 8) bytes (1, or 8 when rows are a multiple of 8
  // bytes) so that a 256-unit box is 1 << box_lbw bytes wide; the wrap maps
  // count bytes.  Boxes are stage_rows high, or one row for the *_row maps.
  CUtensorMap tmap;
  CUtensorMap tmap_row;
  CUtensorMap tmap_wrap;
  CUtensorMap tmap_wrap_row;
  const uint8_t *src;
  uint8_t *dst;
  int64_t src_stride;  // bytes
  int64_t dst_stride;  // bytes
  int32_t width, height, channels;  // source size in pixels
  int32_t out_width, out_height;    // destination size in pixels
  int32_t border;
  int32_t border_value;
  int32_t mode;
  int32_t ksize;
  int32_t use_tma;
  // Separable filters: the taps bound every sum so that plain 32-bit (u16,
  // s16) or 16-bit-lane (u8) accumulation cannot overflow, so the
  // saturation of the reference can only act on the final sums.
  int32_t narrow;
  // Taps of the full kernel: wy vertical, wx horizontal.
  int32_t wy[kMaxTaps];
  int32_t wx[kMaxTaps];
  // Arbitrary-size Gaussian (MODE_SIGMA_SAFE only): reproduces which of the
  // reference's vector / scalar paths handled each element.
  int32_t arbitrary;
  int32_t vert_saturates;
  int32_t arb_border_len;
  // Tiling (see plan_tiles): threads per CTA, rows per tile, rows per TMA
  // stage, stages in the ring, halo chunks per side, strips across a row.
  int32_t threads;
  int32_t tile_rows;
  int32_t stage_rows;
  int32_t stages;
  int32_t halo_chunks;
  int32_t strips;
  int32_t row_tiles;
  // Bands 0 .. big_bands-1 are tile_rows + block_out_rows rows high, the
  // others tile_rows; the last band ends at out_height.
  int32_t big_bands;
  int32_t strip_out_bytes;  // destination bytes produced per strip
  int32_t box_lbw;          // log2 of the span box width in bytes (8 or 11)
};

// One-channel 16-bit 5x5 separable filters (csrc/sep16.cu): a warp strip
// is 32 lanes x 8 elements, of which kSep16Lanes lanes produce output; a
// warp item is (strip, band of at most kSep16MaxBand destination rows).
constexpr int kSep16Lanes = 30;
constexpr int kSep16MaxBand = 15;  // destination rows of a band

struct Sep16Job {
  const uint8_t *src;
  uint8_t *dst;
  int64_t src_stride, dst_stride;  // bytes
  int32_t w, h, border, border_value;
  float kx[5], ky[5];
  int32_t strips, bands;  // warp items: strips x bands, band-major
  int32_t band_q, band_r;  // band b has band_q + (b < band_r) rows
  int32_t edge_every;      // items t with t % edge_every == 0 compute edge elements:
  int32_t edge_per;        // passes [t / edge_every * edge_per, + edge_per) of 32
};

// Four-channel u8 Gaussians, 3x3 / 5x5 / 7x7 generated kernels summing to
// 256 (csrc/gauss8.cu): a warp strip is 32 lanes x 4 pixels, of which
// kGauss8Lanes lanes produce output; a warp item is (strip, band of at most
// kGauss8MaxBand destination rows).
constexpr int kGauss8Lanes = 30;
constexpr int kGauss8MaxBand = 14;

struct Gauss8Job {
  const uint8_t *src;
  uint8_t *dst;
  int64_t src_stride, dst_stride;  // bytes
  int32_t w, h, border, border_value;
  uint32_t w8[7];          // the full kernel (symmetric), K entries
  int32_t strips, bands;   // warp items: strips x bands, band-major
  int32_t band_q, band_r;  // band b has band_q + (b < band_r) rows
  int32_t item_end;        // batch tables: items of this and the earlier entries
};

// Blur-and-downsample levels (csrc/pyramid.cu).  One entry is one level of
// one image: src (w x h) -> dst ((w+1)/2 x (h+1)/2), computed in warp items:
// first its edge tasks (32 edge elements each), then (strip of 32 lanes of
// source bytes, band of at most kPyrBandRows destination rows).  Entries are
// grouped in phases: every entry of a phase depends only on earlier phases
// (level l of every image is phase l - 1), and the kernel separates phases
// with a grid-wide barrier.
constexpr int kPyrBandRows = 8;
constexpr int kPyrMaxPhases = 32;
constexpr int kPyrInline = 8;  // entries carried in the launch parameters

struct PyrEntry {
  const uint8_t *src;
  uint8_t *dst;
  int64_t src_stride, dst_stride;
  int32_t w, h, ow, oh;
  int32_t strips, bands;   // band items: strips x bands (none for an unaligned source)
  int32_t band_q, band_r;  // band b has band_q + (b < band_r) destination rows
  int32_t edge_items;      // the entry's first items
  int32_t item_end;        // warp items of its phase up to and including this entry
  int32_t border, border_value;
};

struct PyrLaunch {
  const PyrEntry *entries;  // device table, or nullptr: inline_entries
  PyrEntry inline_entries[kPyrInline];
  int32_t phase_begin[kPyrMaxPhases + 1];  // entries of phase p: [phase_begin[p], phase_begin[p+1])
  int32_t phases;
  int32_t channels;
  unsigned *barrier;  // zero at launch when phases > 1
  int *err_flag;      // set when a barrier wait hits its limit
};

// One entry of a batched work-list: tile (strip, band) of job `job`.
struct BatchTile {
  uint32_t job;
  uint16_t strip, band;
};

// Generic per-element Gaussian (any odd size up to 255).
struct GenericJob {
  const uint8_t *src;
  uint8_t *dst;
  int64_t src_stride, dst_stride;
  int32_t width, height, channels;
  int32_t border, border_value;
  int32_t ksize;
  int32_t arbitrary;       // reproduce the arbitrary-size path's rounding choices
  int32_t vert_saturates;  // arbitrary path: width*channels >= 16
  int32_t arb_border_len;  // arbitrary path: ceil8(channels * (ksize / 2))
  int32_t v_const;         // vertical result of a column lying in a CONSTANT border
  uint8_t half[128];       // half kernel, half[ksize/2] is the centre weight
};

// Median blur (csrc/median.cu): element type, window size K, border.
enum MedianElem : int32_t {
  MEDIAN_S8 = 0,
  MEDIAN_U8,
  MEDIAN_U16,
  MEDIAN_S16,
  MEDIAN_U32,
  MEDIAN_S32,
  MEDIAN_F32,
};

struct MedianJob {
  const uint8_t *src;
  uint8_t *dst;
  int64_t src_stride, dst_stride;  // bytes
  int32_t width, height, channels, ksize, border, elem;
};

}  // namespace kcv
