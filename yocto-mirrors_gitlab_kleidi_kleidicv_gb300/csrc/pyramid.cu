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
// channels) and a band of kPyrBandRows destination rows, and streams down the
// band's 2 * kPyrBandRows + 3 source rows with no shared memory:
//  * each lane loads its B bytes of a row with vector loads; the few words its
//    taps need beyond them come from the neighbouring lanes by shuffle (lanes
//    0 and 31 load them).  Only bytes inside the row are read (word or byte
//    loads for lanes at the row's ends, and for every lane of a source that
//    vector loads cannot address), and only destination pixels whose five
//    source columns lie inside the row are stored: X in [1, (w - 3) / 2];
//  * horizontal pass: for one to three channels every destination element is
//    a chain of dp4a over the words its five taps fall in (weights [1 4 6 4 1]
//    placed at the taps' byte positions, known at compile time); for four
//    channels the words split into packed 16-bit lanes (channels 0/2 and 1/3)
//    and the taps are whole words;
//  * vertical pass: the horizontal sums of the last three source rows stay in
//    registers as packed 16-bit pairs, and each destination row adds two new
//    rows: a + e + 4 (b + d) + 6 c + 128 per lane, whose high bytes are the
//    destination bytes.
// The source rows of the next destination row are in flight while the
// current one is computed.  The remaining pixels of each row (X = 0 and the
// last one or two) are edge tasks of the same phase: one lane per (row,
// element), its 25 border-mapped source bytes loaded independently.
//
// A pyramid is one launch: each level of each image is a phase, and phases
// are separated by a grid-wide barrier (every CTA resident: cooperative
// launch).  Level l + 1 reads level l right after it was written, mostly from
// L2, through loads that bypass L1.  Every barrier wait is bounded; on expiry
// the kernel sets the error flag and returns.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "launch.h"
#include "sepfused.cuh"

namespace kcv {

namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr uint64_t kBarrierLimitNs = 2000000000ull;

// Lane geometry for C channels.
template <int C>
struct LaneGeo {
  static constexpr int B = C == 3 ? 24 : 16;  // source bytes of a lane
  static constexpr int NW = B / 4;            // its words
  static constexpr int HL = C >= 3 ? 2 : 1;   // words its taps reach to the left
  static constexpr int NT = HL + NW + 1;      // tap window: HL, own words, one to the right
  static constexpr int OUT = B / 2;           // destination bytes of a lane
  static constexpr int NH = OUT / 2;          // packed 16-bit pairs of sums
};

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
__device__ __forceinline__ uint32_t ld32(const uint8_t *p) {
  uint32_t v;
  if (FRESH)
    asm("ld.global.cg.u32 %0, [%1];" : "=r"(v) : "l"(p));
  else
    asm("ld.global.nc.u32 %0, [%1];" : "=r"(v) : "l"(p));
  return v;
}

template <bool FRESH>
__device__ __forceinline__ uint2 ld64(const uint8_t *p) {
  uint2 v;
  if (FRESH)
    asm("ld.global.cg.v2.u32 {%0, %1}, [%2];" : "=r"(v.x), "=r"(v.y) : "l"(p));
  else
    asm("ld.global.nc.v2.u32 {%0, %1}, [%2];" : "=r"(v.x), "=r"(v.y) : "l"(p));
  return v;
}

template <bool FRESH>
__device__ __forceinline__ uint4 ld128(const uint8_t *p) {
  uint4 v;
  if (FRESH)
    asm("ld.global.cg.v4.u32 {%0, %1, %2, %3}, [%4];"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "l"(p));
  else
    asm("ld.global.nc.v4.u32 {%0, %1, %2, %3}, [%4];"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "l"(p));
  return v;
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

// Per-lane constants of one (entry, strip).
struct LaneCtx {
  const uint8_t *src;
  int64_t src_stride;
  long e0;      // first source element (byte) of the lane
  long wc;      // source row bytes
  int w, h, border;
  uint32_t bv;  // CONSTANT border byte
  bool live;    // the lane's window reaches inside the row
  bool fast;    // vector loads: aligned source, tap window inside the row
  bool al4;     // 4-byte aligned source rows
};

// The tap window of source row r (before border mapping): own words at
// t[HL ..], the left words at t[0 .. HL-1], the right word at t[NT-1].  Fast
// lanes other than 0 and 31 leave their left/right words to the shuffle in
// hsums().  Lanes past the row's end leave t as it is.
template <int C, bool FRESH>
__device__ __forceinline__ void load_row(const LaneCtx &lc, int r, int lane, uint32_t (&t)[LaneGeo<C>::NT]) {
  using G = LaneGeo<C>;
  const int y = map_index(r, lc.h, lc.border);
  if (y < 0) {  // a CONSTANT border row: the whole window is the border value
#pragma unroll
    for (int k = 0; k < G::NT; ++k) t[k] = lc.bv * 0x01010101u;
    return;
  }
  const uint8_t *row = lc.src + static_cast<int64_t>(y) * lc.src_stride;
  if (lc.fast) {
    const uint8_t *p = row + lc.e0;
    if constexpr (C == 3) {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const uint2 v = ld64<FRESH>(p + 8 * k);
        t[G::HL + 2 * k] = v.x;
        t[G::HL + 2 * k + 1] = v.y;
      }
    } else {
      const uint4 v = ld128<FRESH>(p);
      t[G::HL] = v.x;
      t[G::HL + 1] = v.y;
      t[G::HL + 2] = v.z;
      t[G::HL + 3] = v.w;
    }
    if (lane == 0) {
      if constexpr (G::HL == 2) {
        const uint2 v = ld64<FRESH>(p - 8);
        t[0] = v.x;
        t[1] = v.y;
      } else {
        t[0] = ld32<FRESH>(p - 4);
      }
    } else if (lane == 31) {
      t[G::NT - 1] = ld32<FRESH>(p + G::B);
    }
  } else if (lc.live) {
    // Lanes at the row's ends and unaligned sources: the window's bytes that
    // lie inside the row (others 0: no stored pixel reads them), whole words
    // where possible.
    const long x0 = lc.e0 - 4 * G::HL;
#pragma unroll
    for (int k = 0; k < G::NT; ++k) {
      const long x = x0 + 4 * k;
      if (lc.al4 && x >= 0 && x + 4 <= lc.wc) {
        t[k] = ld32<FRESH>(row + x);
      } else {
        uint32_t b[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) b[i] = (x + i >= 0 && x + i < lc.wc) ? ld8<FRESH>(row + x + i) : 0u;
        t[k] = b[0] | (b[1] << 8) | (b[2] << 16) | (b[3] << 24);
      }
    }
  }
}

// Horizontal sums of one source row for the lane's OUT destination elements,
// as NH packed 16-bit pairs (sums <= 4080).
template <int C>
__device__ __forceinline__ void hsums(const LaneCtx &lc, int lane, uint32_t (&t)[LaneGeo<C>::NT],
                                      uint32_t (&hs)[LaneGeo<C>::NH]) {
  using G = LaneGeo<C>;
  // Neighbour words: the left lane's last HL words, the right lane's first.
  uint32_t up[G::HL];
#pragma unroll
  for (int k = 0; k < G::HL; ++k) up[k] = __shfl_up_sync(0xffffffffu, t[G::NW + k], 1);
  const uint32_t dn = __shfl_down_sync(0xffffffffu, t[G::HL], 1);
  if (lc.fast) {
    if (lane != 0) {
#pragma unroll
      for (int k = 0; k < G::HL; ++k) t[k] = up[k];
    }
    if (lane != 31) t[G::NT - 1] = dn;
  }
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

// One band (kPyrBandRows destination rows) of one strip of one entry.
template <int C, bool FRESH>
__device__ __forceinline__ void run_band(const PyrEntry &e, int strip, int band, int lane) {
  using G = LaneGeo<C>;
  LaneCtx lc;
  lc.src = e.src;
  lc.src_stride = e.src_stride;
  lc.w = e.w;
  lc.h = e.h;
  lc.border = e.border;
  lc.bv = static_cast<uint32_t>(e.border_value) & 0xFFu;
  lc.wc = static_cast<long>(e.w) * C;
  lc.e0 = (static_cast<long>(strip) * 32 + lane) * G::B;
  lc.live = lc.e0 - 4 * G::HL < lc.wc;
  const uintptr_t sa = reinterpret_cast<uintptr_t>(e.src) | static_cast<uintptr_t>(e.src_stride);
  lc.al4 = (sa & 3) == 0;
  lc.fast = (sa & (C == 3 ? 7 : 15)) == 0 && lc.e0 >= 4 * G::HL && lc.e0 + G::B + 4 <= lc.wc;

  // Stored: destination elements of pixels [1, (w - 3) / 2].
  const long oe = lc.e0 / 2;  // first destination element of the lane
  const long olo = C, ohi = e.w >= 3 ? static_cast<long>((e.w - 3) / 2 + 1) * C : 0;
  const bool stores = oe + G::OUT > olo && oe < ohi;
  const uintptr_t smask = C == 3 ? 3 : 7;
  const bool full_store =
      oe >= olo && oe + G::OUT <= ohi &&
      ((reinterpret_cast<uintptr_t>(e.dst) | static_cast<uintptr_t>(e.dst_stride)) & smask) == 0;

  const int Y0 = band * kPyrBandRows;
  const int Y1 = min(Y0 + kPyrBandRows, e.oh);
  // Horizontal sums of source rows 2Y - 2, 2Y - 1, 2Y (a, b, c) and the raw
  // windows of rows 2Y + 1, 2Y + 2 (r1, r2).
  uint32_t a[G::NH], b[G::NH], c[G::NH];
  uint32_t r1[G::NT], r2[G::NT];
#pragma unroll
  for (int k = 0; k < G::NT; ++k) r1[k] = r2[k] = 0;
  {
    uint32_t s0[G::NT], s1[G::NT], s2[G::NT];
#pragma unroll
    for (int k = 0; k < G::NT; ++k) s0[k] = s1[k] = s2[k] = 0;
    load_row<C, FRESH>(lc, 2 * Y0 - 2, lane, s0);
    load_row<C, FRESH>(lc, 2 * Y0 - 1, lane, s1);
    load_row<C, FRESH>(lc, 2 * Y0, lane, s2);
    load_row<C, FRESH>(lc, 2 * Y0 + 1, lane, r1);
    load_row<C, FRESH>(lc, 2 * Y0 + 2, lane, r2);
    hsums<C>(lc, lane, s0, a);
    hsums<C>(lc, lane, s1, b);
    hsums<C>(lc, lane, s2, c);
  }
  uint8_t *drow = e.dst + static_cast<int64_t>(Y0) * e.dst_stride + oe;
#pragma unroll 1
  for (int Y = Y0; Y < Y1; ++Y) {
    // The next destination row's two source rows are in flight meanwhile.
    uint32_t n1[G::NT], n2[G::NT];
#pragma unroll
    for (int k = 0; k < G::NT; ++k) n1[k] = n2[k] = 0;
    if (Y + 1 < Y1) {
      load_row<C, FRESH>(lc, 2 * Y + 3, lane, n1);
      load_row<C, FRESH>(lc, 2 * Y + 4, lane, n2);
    }
    uint32_t d[G::NH], ee[G::NH];
    hsums<C>(lc, lane, r1, d);
    hsums<C>(lc, lane, r2, ee);
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
#pragma unroll
    for (int k = 0; k < G::NT; ++k) {
      r1[k] = n1[k];
      r2[k] = n2[k];
    }
  }
}

// Edge task `task` of entry e: destination element (Y, X, ch) for the edge
// pixels X = 0 and X in [max(1, (w - 3) / 2 + 1), ow).
template <int C, bool FRESH>
__device__ __forceinline__ void edge_task(const PyrEntry &e, int task) {
  const int xr = e.w >= 3 ? (e.w - 3) / 2 : 0;  // last interior pixel (0: none)
  const int xs = xr + 1 > 1 ? xr + 1 : 1;       // first right-edge pixel
  const int per_row = C * (1 + (e.ow > xs ? e.ow - xs : 0));
  if (task >= per_row * e.oh) return;
  const int Y = task / per_row, q = task - Y * per_row;
  const int p = q / C, ch = q - p * C;
  const int X = p == 0 ? 0 : xs + p - 1;
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

template <int C>
__global__ void __launch_bounds__(kThreads) pyramid_kernel(const __grid_constant__ PyrLaunch L) {
  launch_dependents();
  grid_dependency_wait();  // the source may be the previous call's output
  const PyrEntry *E = L.entries ? L.entries : L.inline_entries;
  const int lane = threadIdx.x & 31;
  const int gwarp = blockIdx.x * kWarps + (threadIdx.x >> 5);
  const int nwarps = gridDim.x * kWarps;
  for (int ph = 0; ph < L.phases; ++ph) {
    if (ph > 0 && !grid_barrier(L.barrier, static_cast<unsigned>(ph), L.err_flag)) return;
    const int e0 = L.phase_begin[ph], e1 = L.phase_begin[ph + 1];
    const int total = E[e1 - 1].item_end;
    for (int t = gwarp; t < total; t += nwarps) {
      // The entry holding item t: the first with item_end > t.
      int lo = e0, hi = e1 - 1;
      while (lo < hi) {
        const int mid = (lo + hi) / 2;
        if (E[mid].item_end > t) hi = mid;
        else lo = mid + 1;
      }
      const PyrEntry &en = E[lo];
      const int local = t - (lo > e0 ? E[lo - 1].item_end : 0);
      if (local < en.main_items) {
        const int band = local / en.strips, strip = local - band * en.strips;
        if (ph == 0)
          run_band<C, false>(en, strip, band, lane);
        else
          run_band<C, true>(en, strip, band, lane);
      } else {
        const int task = (local - en.main_items) * 32 + lane;
        if (ph == 0)
          edge_task<C, false>(en, task);
        else
          edge_task<C, true>(en, task);
      }
    }
  }
}

template <int C>
cudaError_t launch_c(const PyrLaunch &L, int sm_count, cudaStream_t stream) {
  auto kern = pyramid_kernel<C>;
  int occ = 0;
  cudaError_t err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, kThreads, 0);
  if (err != cudaSuccess) return err;
  const PyrEntry *E = L.entries ? nullptr : L.inline_entries;
  long most = 1;
  if (E) {
    for (int ph = 0; ph < L.phases; ++ph)
      most = std::max<long>(most, E[L.phase_begin[ph + 1] - 1].item_end);
  } else {
    most = 1L << 40;  // device table: the caller sized the phases
  }
  const long resident = static_cast<long>(std::max(occ, 1)) * std::max(sm_count, 1);
  const int grid = static_cast<int>(std::max(1L, std::min(resident, (most + kWarps - 1) / kWarps)));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(static_cast<unsigned>(grid));
  cfg.blockDim = dim3(kThreads);
  cfg.dynamicSmemBytes = 0;
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
               int h, int channels, int border, int border_value) {
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
  // A strip makes 32 lanes x (8, or 12 for three channels) destination bytes.
  const long strip_out = 32L * (channels == 3 ? 12 : 8);
  const long owc = static_cast<long>(e.ow) * channels;
  e.strips = static_cast<int32_t>((owc + strip_out - 1) / strip_out);
  e.main_items = e.strips * ((e.oh + kPyrBandRows - 1) / kPyrBandRows);
  // Edge pixels per destination row: X = 0 and X >= max(1, (w - 3) / 2 + 1).
  const int xr = w >= 3 ? (w - 3) / 2 : 0;
  const int xs = xr + 1 > 1 ? xr + 1 : 1;
  const long per_row = static_cast<long>(channels) * (1 + (e.ow > xs ? e.ow - xs : 0));
  e.item_end = e.main_items + static_cast<int32_t>((per_row * e.oh + 31) / 32);
}

}  // namespace kcv
