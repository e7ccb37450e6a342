// blur_and_downsample_u8 and image pyramids (sm_103a).
//
// out[Y][X] = (sum_i sum_j c_i c_j src[b(2Y+i-2)][b(2X+j-2)] + 128) >> 8 per
// channel, c = [1 4 6 4 1] (kleidicv/src/filters/blur_and_downsample_neon.cpp:
// 128-177: a u16 vertical pass on the even rows, then a u16 horizontal pass on
// the even columns).  Every partial sum is exact (at most 65280 + 128), so the
// two passes may run in either order: this kernel filters rows first.
// Destination size ((w+1)/2, (h+1)/2).
//
// A warp owns a strip of 32 lanes x B source bytes (B = 16, or 24 for three
// channels) and a band of at most kPyrBandRows destination rows:
//  * it requests the band's 2 * rows + 3 source rows at once: the strip's
//    bytes plus a 16-byte chunk on either side, as 16-byte cp.async chunks
//    spread over the lanes, into the warp's shared-memory rows, in copy
//    groups of five rows that are filtered as they land;
//  * horizontal pass: each lane reads its tap window (its B bytes and the
//    words around them) from the staged row.  For one to three channels every
//    destination element is a chain of dp4a over the words its five taps fall
//    in (weights [1 4 6 4 1] placed at the taps' byte positions, known at
//    compile time); for four channels the words split into packed 16-bit lanes
//    (channels 0/2 and 1/3) and the taps are whole words;
//  * vertical pass: the horizontal sums of the last three source rows stay in
//    registers as packed 16-bit pairs, and each destination row adds two new
//    rows: a + e + 4 (b + d) + 6 c + 128 per lane, whose high bytes are the
//    destination bytes.
// Only aligned 16-byte blocks that lie wholly inside the row are copied.  With
// an unaligned base or stride each staged row starts at the aligned block
// below the strip's first byte, and the lanes shift their tap windows by that
// row's misalignment (a funnel shift of the staged words).  Only destination
// pixels whose five source columns lie inside the copied blocks of every row
// are stored: X in [xl, xr] (xl = 1 for aligned rows; unaligned rows leave up
// to 15 bytes at either end uncovered).  The remaining pixels of each row are
// edge tasks of the same phase, scheduled first: one lane per (row, element),
// its 25 border-mapped source bytes loaded independently.
//
// A pyramid is one launch: each level of each image is a phase, and phases
// are separated by a grid-wide barrier (every CTA resident: cooperative
// launch).  Level l + 1 reads level l right after it was written, mostly from
// L2, through copies and loads that bypass L1.  Every barrier wait is bounded;
// on expiry the kernel sets the error flag and returns.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "launch.h"
#include "resident.cuh"
#include "sepfused.cuh"

namespace kcv {

namespace {

constexpr int kThreads = 128;
constexpr int kWarps = kThreads / 32;
constexpr int kStageRows = 2 * kPyrBandRows + 3;
constexpr int kGroups = (kStageRows + 4) / 5;  // copy groups of five rows: 4
constexpr uint64_t kBarrierLimitNs = 2000000000ull;
constexpr int kPyrSearchEntries = 512;  // phases with more entries search in global memory

// Lane geometry for C channels.
template <int C>
struct LaneGeo {
  static constexpr int B = C == 3 ? 24 : 16;  // source bytes of a lane
  static constexpr int NW = B / 4;            // its words
  static constexpr int HL = C >= 3 ? 2 : 1;   // words its taps reach to the left
  static constexpr int NT = HL + NW + 1;      // tap window: HL, own words, one to the right
  static constexpr int OUT = B / 2;           // destination bytes of a lane
  static constexpr int NH = OUT / 2;          // packed 16-bit pairs of sums
  static constexpr int SPAN = 32 * B;         // strip bytes
  // Staged 16-byte chunks of a row: the strip +- 16 bytes, and one more for
  // a row start up to 15 bytes past the first chunk's boundary.
  static constexpr int CHUNKS = SPAN / 16 + 3;
  static constexpr int ROW = CHUNKS * 16;       // staged row bytes
  static constexpr int WARP_STAGE = kStageRows * ROW;
};

template <int C>
constexpr int smem_bytes() {
  return kWarps * LaneGeo<C>::WARP_STAGE;
}

// dp4a weight word of window word q (relative to the lane's first word) for
// destination element j of the lane (one to three channels): the tap weights
// at the byte positions of the taps that fall in word q.  Element j has
// channel j % C and source centre 2 C (j / C) + j % C.
__host__ __device__ constexpr uint32_t tap_word(int c, int j, int q) {
  const int centre = 2 * c * (j / c) + j % c;
  uint32_t w = 0;
  for (int d = -2; d <= 2; ++d) {
    const int pos = centre + c * d;
    const int wq = floor_div(pos, 4);
    const uint32_t coef = d == 0 ? 6u : (d == 1 || d == -1 ? 4u : 1u);
    if (wq == q) w += coef << (8 * (pos - 4 * wq));
  }
  return w;
}

template <bool FRESH>
__device__ __forceinline__ uint32_t ld8(const uint8_t *p) {
  uint16_t v;
  if (FRESH)
    asm("ld.global.cg.u8 %0, [%1];" : "=h"(v) : "l"(p));
  else
    asm("ld.global.nc.u8 %0, [%1];" : "=h"(v) : "l"(p));
  return v;
}

// cp.async.cg goes through L2 only: safe for a source written earlier in the
// same launch.  No "memory" clobber: nothing reads the slot before the wait.
__device__ __forceinline__ void cp_async16p(uint32_t dst, const void *src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src));
}
__device__ __forceinline__ void cp_async_commit_p() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait_p() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
// Waits until at most `pending` copy groups are outstanding, then makes the
// warp's copies visible to all its lanes.
__device__ __forceinline__ void wait_groups(int pending) {
  switch (pending) {
    case 0: cp_async_wait_p<0>(); break;
    case 1: cp_async_wait_p<1>(); break;
    case 2: cp_async_wait_p<2>(); break;
    default: cp_async_wait_p<3>(); break;
  }
  __syncwarp();
}

__device__ __forceinline__ uint32_t ld_acquire_u32(const unsigned *p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Grid-wide barrier number `epoch` (1, 2, ...): every CTA adds one to the
// counter and waits until all gridDim.x CTAs have, at most kBarrierLimitNs.
__device__ bool grid_barrier(unsigned *count, unsigned epoch, int *err_flag) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();  // this CTA's outputs before its arrival
    atomicAdd(count, 1u);
    const unsigned target = epoch * gridDim.x;
    const uint64_t start = global_timer_ns();
    int good = 1;
    while (ld_acquire_u32(count) < target) {
      if (global_timer_ns() - start > kBarrierLimitNs) {
        atomicOr(err_flag, 1);
        good = 0;
        break;
      }
      __nanosleep(100);
    }
    ok = good;
  }
  __syncthreads();
  return ok != 0;
}

// Horizontal sums of the lane's tap window t (NT source words) for its OUT
// destination elements, as NH packed 16-bit pairs (sums <= 4080).
template <int C>
__device__ __forceinline__ void hsums_words(const uint32_t (&t)[LaneGeo<C>::NT], uint32_t (&hs)[LaneGeo<C>::NH]) {
  using G = LaneGeo<C>;
  if constexpr (C == 4) {
    // Window word k is pixel k - 2 of the lane; destination pixel m is
    // centred on pixel 2m: its taps are words 2m .. 2m + 4.
    uint32_t lo[G::NT], hi[G::NT];
#pragma unroll
    for (int k = 0; k < G::NT; ++k) {
      lo[k] = t[k] & 0x00FF00FFu;            // channels 0, 2
      hi[k] = __byte_perm(t[k], 0u, 0x4341);  // channels 1, 3
    }
#pragma unroll
    for (int m = 0; m < 2; ++m) {
      const int i = 2 * m;
      hs[2 * m] = lo[i] + lo[i + 4] + 4u * (lo[i + 1] + lo[i + 3]) + 6u * lo[i + 2];
      hs[2 * m + 1] = hi[i] + hi[i + 4] + 4u * (hi[i + 1] + hi[i + 3]) + 6u * hi[i + 2];
    }
  } else {
    uint32_t o[G::OUT];
    static_for<0, G::OUT>([&](auto jc) {
      constexpr int J = decltype(jc)::value;
      uint32_t acc = 0;
      static_for<0, G::NT>([&](auto kc) {
        constexpr int K = decltype(kc)::value;
        constexpr uint32_t wt = tap_word(C, J, K - G::HL);
        if constexpr (wt != 0) acc = __dp4a(t[K], wt, acc);
      });
      o[J] = acc;
    });
#pragma unroll
    for (int k = 0; k < G::NH; ++k) hs[k] = __byte_perm(o[2 * k], o[2 * k + 1], 0x5410);
  }
}

// Horizontal sums of one staged source row.  `row` is the staged row, `off`
// the byte offset of the lane's tap window in it (a multiple of 4), `mis` the
// row's misalignment (0..15: the staged bytes start `mis` bytes before the
// row byte that `off` counts from).
template <int C, bool ALIGNED>
__device__ __forceinline__ void hsums(const uint8_t *row, int off, int mis, uint32_t (&hs)[LaneGeo<C>::NH]) {
  using G = LaneGeo<C>;
  uint32_t t[G::NT];
  if constexpr (ALIGNED) {
#pragma unroll
    for (int k = 0; k < G::NT; ++k) t[k] = *reinterpret_cast<const uint32_t *>(row + off + 4 * k);
  } else {
    const uint32_t *q = reinterpret_cast<const uint32_t *>(row + off + (mis & ~3));
    const unsigned sh = 8u * static_cast<unsigned>(mis & 3);
    uint32_t wv[G::NT + 1];
#pragma unroll
    for (int k = 0; k <= G::NT; ++k) wv[k] = q[k];
#pragma unroll
    for (int k = 0; k < G::NT; ++k) t[k] = __funnelshift_r(wv[k], wv[k + 1], sh);
  }
  hsums_words<C>(t, hs);
}

// Interior destination pixels of a level, [first, last] (last < first: none):
// their five source columns lie inside the aligned 16-byte blocks wholly
// inside every row.  Aligned rows: the blocks cover the row's first
// 16 * floor(w c / 16) bytes.  Unaligned rows: at least bytes [15, w c - 15).
struct Interior {
  int first, last;
};
__host__ __device__ inline Interior interior(int w, int c, bool aligned) {
  const long wc = static_cast<long>(w) * c;
  const long covered = aligned ? wc / 16 * 16 : wc - 15;  // bytes [lead, covered) are staged
  const int wsafe = covered > 0 ? static_cast<int>(covered / c) : 0;
  Interior r;
  // Leftmost tap byte 2 c (X - 1) >= lead: X >= 1 (lead 0), else X >= ceil((15 + 2c) / 2c).
  r.first = aligned ? 1 : (14 + 4 * c) / (2 * c);
  // Rightmost tap pixel 2 X + 2 < wsafe.
  r.last = wsafe >= 3 ? (wsafe - 3) / 2 : -1;
  return r;
}

__host__ __device__ inline bool rows_aligned(const uint8_t *src, int64_t stride) {
  return ((reinterpret_cast<uintptr_t>(src) | static_cast<uintptr_t>(stride)) & 15) == 0;
}

// One band of one strip of one entry (ALIGNED: 16-byte aligned base and
// stride).
template <int C, bool FRESH, bool ALIGNED>
__device__ __forceinline__ void run_band(const PyrEntry &e, uint8_t *stage, int strip, int band, int lane) {
  using G = LaneGeo<C>;
  const long wc = static_cast<long>(e.w) * C;
  const long base = static_cast<long>(strip) * G::SPAN - 16;  // row byte of staged chunk 0
  const long e0 = static_cast<long>(strip) * G::SPAN + static_cast<long>(lane) * G::B;
  const int off = static_cast<int>(e0 - 4 * G::HL - base);  // lane's tap window in the staged row
  const uint32_t bv4 = (static_cast<uint32_t>(e.border_value) & 0xFFu) * 0x01010101u;

  const int rows = e.band_q + (band < e.band_r ? 1 : 0);
  const int Y0 = band * e.band_q + min(band, e.band_r);
  const int nrows = 2 * rows + 3;  // source rows 2 Y0 - 2 .. 2 Y1

  // Copies: row rr of the stage holds source row 2 Y0 - 2 + rr from row byte
  // base - mis (mis: the row start's misalignment, 0 when aligned and for a
  // constant-border row); each lane copies chunks lane and lane + 32 of it,
  // the aligned blocks wholly inside the row.  The misalignments are kept as
  // 4-bit fields for the reads.
  const uint32_t sbase = static_cast<uint32_t>(__cvta_generic_to_shared(stage));
  uint64_t mis_lo = 0;  // rows 0 .. 15
  uint32_t mis_hi = 0;  // rows 16 .. 18
  int rr = 0;
#pragma unroll
  for (int grp = 0; grp < kGroups; ++grp) {
#pragma unroll 1
    for (; rr < min(nrows, 5 * grp + 5); ++rr) {
      const int y = map_index(2 * Y0 - 2 + rr, e.h, e.border);
      const uint8_t *srow = y < 0 ? e.src : e.src + static_cast<int64_t>(y) * e.src_stride;
      const int mis = (ALIGNED || y < 0) ? 0 : static_cast<int>(reinterpret_cast<uintptr_t>(srow) & 15);
      if constexpr (!ALIGNED) {
        if (rr < 16) mis_lo |= static_cast<uint64_t>(mis) << (4 * rr);
        else mis_hi |= static_cast<uint32_t>(mis) << (4 * (rr - 16));
      }
#pragma unroll
      for (int k = lane; k < G::CHUNKS; k += 32) {
        const long x = base + 16L * k - mis;
        if (y < 0) {
          *reinterpret_cast<uint4 *>(stage + rr * G::ROW + 16 * k) = make_uint4(bv4, bv4, bv4, bv4);
        } else if (x >= 0 && x + 16 <= wc) {
          cp_async16p(sbase + rr * G::ROW + 16 * k, srow + x);
        }
      }
    }
    cp_async_commit_p();
  }
  auto mis_of = [&](int row) -> int {
    if constexpr (ALIGNED) return 0;
    return row < 16 ? static_cast<int>((mis_lo >> (4 * row)) & 15) : static_cast<int>((mis_hi >> (4 * (row - 16))) & 15);
  };

  // Stored: destination elements of pixels [xl, xr].
  const Interior in = interior(e.w, C, ALIGNED);
  const long oe = e0 / 2;  // first destination element of the lane
  const long olo = static_cast<long>(in.first) * C, ohi = static_cast<long>(in.last + 1) * C;
  const bool stores = oe + G::OUT > olo && oe < ohi;
  const uintptr_t smask = C == 3 ? 3 : 7;
  const bool full_store =
      oe >= olo && oe + G::OUT <= ohi &&
      ((reinterpret_cast<uintptr_t>(e.dst) | static_cast<uintptr_t>(e.dst_stride)) & smask) == 0;

  uint32_t a[G::NH], b[G::NH], c[G::NH];
  wait_groups(kGroups - 1);  // group 0: rows 0 .. 4
  hsums<C, ALIGNED>(stage, off, mis_of(0), a);
  hsums<C, ALIGNED>(stage + G::ROW, off, mis_of(1), b);
  hsums<C, ALIGNED>(stage + 2 * G::ROW, off, mis_of(2), c);
  uint8_t *drow = e.dst + static_cast<int64_t>(Y0) * e.dst_stride + oe;
#pragma unroll 1
  for (int r = 0; r < rows; ++r) {
    // Destination row r reads stage rows 2r + 3 and 2r + 4: group (2r + 4) / 5.
    wait_groups(max(0, kGroups - 1 - (2 * r + 4) / 5));
    uint32_t d[G::NH], ee[G::NH];
    hsums<C, ALIGNED>(stage + (2 * r + 3) * G::ROW, off, mis_of(2 * r + 3), d);
    hsums<C, ALIGNED>(stage + (2 * r + 4) * G::ROW, off, mis_of(2 * r + 4), ee);
    uint32_t s[G::NH];
#pragma unroll
    for (int k = 0; k < G::NH; ++k) s[k] = a[k] + ee[k] + 0x00800080u + 4u * (b[k] + d[k]) + 6u * c[k];
    // Destination bytes: the high byte of every 16-bit lane.
    uint32_t ow[G::NH / 2];
#pragma unroll
    for (int k = 0; k < G::NH / 2; ++k)
      ow[k] = __byte_perm(s[2 * k], s[2 * k + 1], C == 4 ? 0x7351 : 0x7531);
    if (stores) {
      if (full_store) {
        if constexpr (C == 3) {
          uint32_t *q = reinterpret_cast<uint32_t *>(drow);
          q[0] = ow[0];
          q[1] = ow[1];
          q[2] = ow[2];
        } else {
          *reinterpret_cast<uint2 *>(drow) = make_uint2(ow[0], ow[1]);
        }
      } else {
#pragma unroll
        for (int k = 0; k < G::OUT; ++k)
          if (oe + k >= olo && oe + k < ohi) drow[k] = static_cast<uint8_t>(ow[k >> 2] >> (8 * (k & 3)));
      }
    }
    drow += e.dst_stride;
#pragma unroll
    for (int k = 0; k < G::NH; ++k) {
      a[k] = c[k];
      b[k] = d[k];
      c[k] = ee[k];
    }
  }
  // The stage is rewritten by the warp's next item only after every lane
  // has read it.
  __syncwarp();
}

// Edge pixels of a row: X in [0, xl) and [xs, ow), with xl = min(first, ow)
// and xs = max(last + 1, xl).
struct EdgeSplit {
  int xl, xs, per_row;  // per_row: edge elements of a destination row
};
__host__ __device__ inline EdgeSplit edge_split(int w, int ow, int c, bool aligned) {
  const Interior in = interior(w, c, aligned);
  EdgeSplit s;
  s.xl = in.first < ow ? in.first : ow;
  s.xs = in.last + 1 > s.xl ? in.last + 1 : s.xl;
  s.per_row = c * (s.xl + (ow > s.xs ? ow - s.xs : 0));
  return s;
}

// Edge task `task` of entry e: destination element (Y, X, ch) of an edge
// pixel.
template <int C, bool FRESH>
__device__ __forceinline__ void edge_task(const PyrEntry &e, int task) {
  const EdgeSplit sp = edge_split(e.w, e.ow, C, rows_aligned(e.src, e.src_stride));
  const int per_row = sp.per_row;
  if (task >= per_row * e.oh) return;
  const int Y = task / per_row, q = task - Y * per_row;
  const int p = q / C, ch = q - p * C;
  const int X = p < sp.xl ? p : sp.xs + p - sp.xl;
  const uint32_t bv = static_cast<uint32_t>(e.border_value) & 0xFFu;
  const uint8_t *rows[5];
  long cols[5];
#pragma unroll
  for (int d = 0; d < 5; ++d) {
    const int my = map_index(2 * Y + d - 2, e.h, e.border);
    rows[d] = my < 0 ? nullptr : e.src + static_cast<int64_t>(my) * e.src_stride;
    const int mc = map_index(2 * X + d - 2, e.w, e.border);
    cols[d] = mc < 0 ? -1 : static_cast<long>(mc) * C + ch;
  }
  uint32_t v[5][5];
#pragma unroll
  for (int r = 0; r < 5; ++r)
#pragma unroll
    for (int c = 0; c < 5; ++c) v[r][c] = (rows[r] && cols[c] >= 0) ? ld8<FRESH>(rows[r] + cols[c]) : bv;
  const uint32_t wt[5] = {1, 4, 6, 4, 1};
  uint32_t sum = 128;
#pragma unroll
  for (int r = 0; r < 5; ++r) {
    const uint32_t hsum = v[r][0] + v[r][4] + 4u * (v[r][1] + v[r][3]) + 6u * v[r][2];
    sum += wt[r] * hsum;
  }
  e.dst[static_cast<int64_t>(Y) * e.dst_stride + static_cast<long>(X) * C + ch] = static_cast<uint8_t>(sum >> 8);
}

template <int C, bool FRESH>
__device__ __forceinline__ void run_item(const PyrEntry &en, uint8_t *stage, int local, int lane) {
  if (local < en.edge_items) {
    edge_task<C, FRESH>(en, local * 32 + lane);
  } else {
    // Strips rotate by 7 per band: a warp's items do not all land on the
    // strips at the row's ends.
    const int m = local - en.edge_items;
    const int band = m / en.strips, q = m - band * en.strips;
    const int strip = static_cast<int>((q + 7L * band) % en.strips);
    if (rows_aligned(en.src, en.src_stride))
      run_band<C, FRESH, true>(en, stage, strip, band, lane);
    else
      run_band<C, FRESH, false>(en, stage, strip, band, lane);
  }
}

template <int C>
__global__ void __launch_bounds__(kThreads) pyramid_kernel(const __grid_constant__ PyrLaunch L) {
  extern __shared__ __align__(16) uint8_t pyr_stage[];
  launch_dependents();
  grid_dependency_wait();  // the source may be the previous call's output
  const PyrEntry *E = L.entries ? L.entries : L.inline_entries;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint8_t *stage = pyr_stage + warp * LaneGeo<C>::WARP_STAGE;
  // Items go round the CTAs first, so that every SM gets the same number.
  const int gwarp = warp * gridDim.x + blockIdx.x;
  const int nwarps = gridDim.x * kWarps;
  // The phase's item boundaries, for the entry search (a table in global
  // memory would make every search a chain of dependent loads).
  __shared__ int ends[kPyrSearchEntries];
  for (int ph = 0; ph < L.phases; ++ph) {
    if (ph > 0 && !grid_barrier(L.barrier, static_cast<unsigned>(ph), L.err_flag)) return;
    const int e0 = L.phase_begin[ph], e1 = L.phase_begin[ph + 1];
    const bool cached = e1 - e0 <= kPyrSearchEntries;
    __syncthreads();  // the previous phase's readers of ends[] are done
    if (cached)
      for (int k = threadIdx.x; k < e1 - e0; k += blockDim.x) ends[k] = E[e0 + k].item_end;
    __syncthreads();
    const int total = E[e1 - 1].item_end;
    for (int t = gwarp; t < total; t += nwarps) {
      // The entry holding item t: the first with item_end > t.
      int lo = e0, hi = e1 - 1;
      while (lo < hi) {
        const int mid = (lo + hi) / 2;
        if ((cached ? ends[mid - e0] : E[mid].item_end) > t) hi = mid;
        else lo = mid + 1;
      }
      const PyrEntry en = E[lo];  // one round of loads, then registers
      const int local = t - (lo > e0 ? (cached ? ends[lo - 1 - e0] : E[lo - 1].item_end) : 0);
      if (ph == 0)
        run_item<C, false>(en, stage, local, lane);
      else
        run_item<C, true>(en, stage, local, lane);
    }
  }
}

template <int C>
int warps_c(int sm_count) {
  int occ = 0;
  if (resident_ctas_per_sm<pyramid_kernel<C>>(kThreads, smem_bytes<C>(), &occ) != cudaSuccess) return 0;
  return occ * std::max(sm_count, 1) * kWarps;
}

template <int C>
cudaError_t launch_c(const PyrLaunch &L, int sm_count, cudaStream_t stream) {
  auto kern = pyramid_kernel<C>;
  const int warps = warps_c<C>(sm_count);
  if (warps == 0) return cudaErrorInvalidValue;
  const PyrEntry *E = L.entries ? nullptr : L.inline_entries;
  long most = 1;
  if (E) {
    for (int ph = 0; ph < L.phases; ++ph)
      most = std::max<long>(most, E[L.phase_begin[ph + 1] - 1].item_end);
  } else {
    most = 1L << 40;  // device table: the caller sized the phases
  }
  const int grid = static_cast<int>(std::max(1L, std::min<long>(warps / kWarps, (most + kWarps - 1) / kWarps)));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(static_cast<unsigned>(grid));
  cfg.blockDim = dim3(kThreads);
  cfg.dynamicSmemBytes = smem_bytes<C>();
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  if (L.phases > 1) {
    // Grid-wide barriers need every CTA resident.
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
  } else {
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
  }
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, L);
}

}  // namespace

int pyramid_warps(int channels, int sm_count) {
  switch (channels) {
    case 1: return warps_c<1>(sm_count);
    case 2: return warps_c<2>(sm_count);
    case 3: return warps_c<3>(sm_count);
    case 4: return warps_c<4>(sm_count);
  }
  return 0;
}

cudaError_t launch_pyramid(const PyrLaunch &L, int sm_count, cudaStream_t stream) {
  if (L.phases > 1) {
    const cudaError_t e = cudaMemsetAsync(L.barrier, 0, sizeof(unsigned), stream);
    if (e != cudaSuccess) return e;
  }
  switch (L.channels) {
    case 1: return launch_c<1>(L, sm_count, stream);
    case 2: return launch_c<2>(L, sm_count, stream);
    case 3: return launch_c<3>(L, sm_count, stream);
    case 4: return launch_c<4>(L, sm_count, stream);
  }
  return cudaErrorInvalidValue;
}

void pyr_entry(PyrEntry &e, const uint8_t *src, int64_t src_stride, uint8_t *dst, int64_t dst_stride, int w,
               int h, int channels, int border, int border_value, int warps) {
  e.border = border;
  e.border_value = border_value;
  e.src = src;
  e.dst = dst;
  e.src_stride = src_stride;
  e.dst_stride = dst_stride;
  e.w = w;
  e.h = h;
  e.ow = (w + 1) / 2;
  e.oh = (h + 1) / 2;
  const bool aligned = rows_aligned(src, src_stride);
  const EdgeSplit sp = edge_split(w, e.ow, channels, aligned);
  // A strip makes 32 lanes x (8, or 12 for three channels) destination bytes;
  // no strips when no pixel is interior.
  const long strip_out = 32L * (channels == 3 ? 12 : 8);
  const long owc = static_cast<long>(e.ow) * channels;
  e.strips = sp.xs > sp.xl ? static_cast<int32_t>((owc + strip_out - 1) / strip_out) : 0;
  // Bands of at most kPyrBandRows rows, as many as give every warp the same
  // number of items.
  long bands = 0;
  if (e.strips > 0) {
    const long min_bands = (e.oh + kPyrBandRows - 1) / kPyrBandRows;
    const long slots = std::max(warps, 1);
    const long per_warp = std::max(1L, (min_bands * e.strips + slots - 1) / slots);
    bands = std::min<long>(e.oh, std::max(min_bands, per_warp * slots / e.strips));
  }
  e.bands = static_cast<int32_t>(bands);
  e.band_q = bands > 0 ? static_cast<int32_t>(e.oh / bands) : 0;
  e.band_r = bands > 0 ? static_cast<int32_t>(e.oh % bands) : 0;
  e.edge_items = static_cast<int32_t>((static_cast<long>(sp.per_row) * e.oh + 31) / 32);
  e.item_end = e.edge_items + static_cast<int32_t>(e.strips * bands);
}

}  // namespace kcv
