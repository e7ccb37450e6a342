// gaussian_blur_u8 on four-channel images with generated 3x3, 5x5 and 7x7
// kernels whose weights sum to 256 (sm_103a).
//
// Arithmetic (kleidicv/src/filters/gaussian_blur_fixed_neon.cpp:501-526 and
// the horizontal pass after it): each vertical sum 128 + sum_t w_t x_t is
// narrowed to u8 by >> 8, then each horizontal sum 128 + sum_t w_t v_t gives
// the destination byte by >> 8.  With weights summing to 256 both sums stay
// below 65536, so two channels share one 32-bit word as 16-bit lanes: a word
// of four channels splits into (channels 0, 2) and (channels 1, 3).  The
// kernel is symmetric, so rows (and pixels) at equal distance from the centre
// are added before their common weight multiplies them: (K - 1) / 2 adds and
// (K + 1) / 2 multiply-adds per lane pair and pass.
//
// A warp owns a strip of 32 lanes x 4 pixels (16 bytes) of a row, of which
// lanes 1..30 produce output and lanes 0 and 31 only supply the horizontal
// halo (up to three pixels) by shuffle, and a band of at most kGauss8MaxBand
// destination rows.  It requests every source row of the band at once (one
// 16-byte cp.async per lane and row into its own shared-memory slots), in
// copy groups of K rows that are filtered as they land, then streams down
// the band: the unpacked rows of the vertical window stay in registers in
// statically indexed slots (the row loop is unrolled by K).  The source rows
// must be 4-byte aligned (whole pixels; other calls take the tiled kernel of
// sepfused.cuh).  With 16-byte aligned rows, lanes whose 4 pixels lie inside the
// row copy them as one 16-byte piece; lanes at the row's ends (left of pixel
// 0, or reaching past the last pixel), and every lane of rows that are not
// 16-byte aligned, copy each of their pixels from its border-mapped column
// with a 4-byte cp.async (the border value for CONSTANT), so every stored
// pixel reads real neighbours and the row ends need no separate pass.  Warps
// whose every lane stores whole 16-byte pieces run a loop without the
// per-pixel store path, which writes 4-byte words where the destination
// allows and bytes otherwise.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "launch.h"
#include "resident.cuh"
#include "sepfused.cuh"

namespace kcv {

namespace {

constexpr int kThreadsG = 128;
constexpr int kWarpsG = kThreadsG / 32;
constexpr int kPix = 4;                            // pixels (16 bytes) per lane
constexpr int kStripPix = kGauss8Lanes * kPix;     // destination pixels per strip
constexpr int kStageRowsMax = kGauss8MaxBand + 6;  // source rows of a band, K <= 7
constexpr int kWarpStage = kStageRowsMax * 32 * 16;
constexpr int kSmemG = kWarpsG * kWarpStage;  // 40960

__device__ __forceinline__ void cp_async16g(uint32_t dst, const void *src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src));
}
__device__ __forceinline__ void cp_async_commit_g() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait_g() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
// Waits until at most `pending` copy groups (0..7) are outstanding.
__device__ __forceinline__ void cp_async_wait_upto(int pending) {
  switch (pending) {
    case 0: cp_async_wait_g<0>(); break;
    case 1: cp_async_wait_g<1>(); break;
    case 2: cp_async_wait_g<2>(); break;
    case 3: cp_async_wait_g<3>(); break;
    case 4: cp_async_wait_g<4>(); break;
    case 5: cp_async_wait_g<5>(); break;
    case 6: cp_async_wait_g<6>(); break;
    default: cp_async_wait_g<7>(); break;
  }
}

template <int K>
struct GaussGeo {
  static constexpr int R = K / 2;
  static constexpr int kStageRows = kGauss8MaxBand + K - 1;
  static constexpr int kGroups = (kStageRows + K - 1) / K;  // copy groups of K rows
};

// One lane's 4 pixels of a row as (channels 0, 2) and (channels 1, 3) words.
__device__ __forceinline__ void unpack4(const uint4 &raw, uint32_t (&lo)[kPix], uint32_t (&hi)[kPix]) {
  const uint32_t w[4] = {raw.x, raw.y, raw.z, raw.w};
#pragma unroll
  for (int p = 0; p < kPix; ++p) {
    lo[p] = w[p] & 0x00FF00FFu;
    hi[p] = __byte_perm(w[p], 0u, 0x4341);
  }
}

// 128 + the symmetric K-tap sum over the packed words a[c - R .. c + R].
template <int K>
__device__ __forceinline__ uint32_t sym_sum(const uint32_t (&wt)[K / 2 + 1], uint32_t centre,
                                            const uint32_t *left, const uint32_t *right) {
  // left[d - 1] and right[d - 1]: the words at distance d.
  uint32_t acc = wt[K / 2] * centre + 0x00800080u;
#pragma unroll
  for (int d = 1; d <= K / 2; ++d) acc += wt[K / 2 - d] * (left[d - 1] + right[d - 1]);
  return acc;
}

// Destination row from the window (its source row y - R in slot S0, y - R + 1
// in S0 + 1, ... modulo K): vertical sums narrowed to u8 lanes, the
// neighbours' halo by shuffle, horizontal sums, destination bytes.
template <int K, int S0>
__device__ __forceinline__ uint4 filter_row8(const uint32_t (&wl)[K][kPix], const uint32_t (&wh)[K][kPix],
                                             const uint32_t (&wt)[K / 2 + 1]) {
  constexpr int R = K / 2;
  constexpr int C = (S0 + R) % K;  // slot of the centre row
  // V[R + p]: vertical results of pixel p of the lane; V[0 .. R-1] and
  // V[R + 4 ..] come from the neighbour lanes.
  uint32_t Vl[kPix + 2 * R], Vh[kPix + 2 * R];
#pragma unroll
  for (int p = 0; p < kPix; ++p) {
    uint32_t ll[R > 0 ? R : 1], lr[R > 0 ? R : 1], hl[R > 0 ? R : 1], hr[R > 0 ? R : 1];
#pragma unroll
    for (int d = 1; d <= R; ++d) {
      ll[d - 1] = wl[(C + K - d) % K][p];
      lr[d - 1] = wl[(C + d) % K][p];
      hl[d - 1] = wh[(C + K - d) % K][p];
      hr[d - 1] = wh[(C + d) % K][p];
    }
    Vl[R + p] = __byte_perm(sym_sum<K>(wt, wl[C][p], ll, lr), 0u, 0x4341);
    Vh[R + p] = __byte_perm(sym_sum<K>(wt, wh[C][p], hl, hr), 0u, 0x4341);
  }
#pragma unroll
  for (int d = 0; d < R; ++d) {
    Vl[d] = __shfl_up_sync(0xffffffffu, Vl[kPix + d], 1);  // left lane's pixel 4 - R + d
    Vh[d] = __shfl_up_sync(0xffffffffu, Vh[kPix + d], 1);
    Vl[R + kPix + d] = __shfl_down_sync(0xffffffffu, Vl[R + d], 1);  // right lane's pixel d
    Vh[R + kPix + d] = __shfl_down_sync(0xffffffffu, Vh[R + d], 1);
  }
  uint32_t o[kPix];
#pragma unroll
  for (int p = 0; p < kPix; ++p) {
    uint32_t ll[R > 0 ? R : 1], lr[R > 0 ? R : 1], hl[R > 0 ? R : 1], hr[R > 0 ? R : 1];
#pragma unroll
    for (int d = 1; d <= R; ++d) {
      ll[d - 1] = Vl[R + p - d];
      lr[d - 1] = Vl[R + p + d];
      hl[d - 1] = Vh[R + p - d];
      hr[d - 1] = Vh[R + p + d];
    }
    const uint32_t sl = sym_sum<K>(wt, Vl[R + p], ll, lr);
    const uint32_t sh = sym_sum<K>(wt, Vh[R + p], hl, hr);
    o[p] = __byte_perm(sl, sh, 0x7351);  // channels 0..3: high bytes of the lanes
  }
  return make_uint4(o[0], o[1], o[2], o[3]);
}

__device__ __forceinline__ void cp_async4g(uint32_t dst, const void *src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(dst), "l"(src));
}

template <int K, bool SIMPLE>
__device__ __forceinline__ void band_loop8(const Gauss8Job &j, const uint4 *stage, int lane, int rows,
                                           uint8_t *d, long e0, bool outputs, bool full_store);

template <int K>
__device__ __forceinline__ void run_band8(const Gauss8Job &j, uint4 *stage, int strip, int band, int lane) {
  using G = GaussGeo<K>;
  constexpr int R = G::R;
  const long e0 = static_cast<long>(strip) * kStripPix + kPix * lane - kPix;  // first pixel of the lane
  // Pixels needed by stored outputs: [-R, w + R).
  const bool live = e0 + kPix > -R && e0 < static_cast<long>(j.w) + R;
  const bool rows16 = ((reinterpret_cast<uintptr_t>(j.src) | static_cast<uintptr_t>(j.src_stride)) & 15) == 0;
  const bool fast = rows16 && e0 >= 0 && e0 + kPix <= j.w;
  // Border lanes: the source column of each pixel (-1: the border value).
  int col[kPix];
#pragma unroll
  for (int k = 0; k < kPix; ++k) col[k] = map_index(static_cast<int>(e0) + k, j.w, j.border);
  const bool outputs = lane >= 1 && lane <= kGauss8Lanes && e0 >= 0 && e0 < j.w;
  const bool full_store =
      outputs && e0 + kPix <= j.w &&
      ((reinterpret_cast<uintptr_t>(j.dst) | static_cast<uintptr_t>(j.dst_stride)) & 15) == 0;
  const uint32_t bv4 = (static_cast<uint32_t>(j.border_value) & 0xFFu) * 0x01010101u;

  const int rows = j.band_q + (band < j.band_r ? 1 : 0);
  const int y0 = band * j.band_q + min(band, j.band_r);
  const int y1 = y0 + rows;
  const int nrows = rows + K - 1;  // source rows y0 - R .. y1 + R - 1
  // Request every source row: slot rr of the lane holds row y0 - R + rr, in
  // groups of K rows ([gK, gK + K); empty groups at the end).
  const uint32_t sbase = static_cast<uint32_t>(__cvta_generic_to_shared(stage + lane));
  if (fast && y0 >= R && y1 + R <= j.h) {
    const uint8_t *g = j.src + static_cast<int64_t>(y0 - R) * j.src_stride + 4 * e0;
    uint32_t a = sbase;
    int rr = 0;
#pragma unroll
    for (int grp = 0; grp < G::kGroups; ++grp) {
#pragma unroll 1
      for (; rr < min(nrows, K * grp + K); ++rr, a += 32 * 16, g += j.src_stride) cp_async16g(a, g);
      cp_async_commit_g();
    }
  } else {
    int rr = 0;
#pragma unroll
    for (int grp = 0; grp < G::kGroups; ++grp) {
#pragma unroll 1
      for (; rr < min(nrows, K * grp + K); ++rr) {
        const int y = map_index(y0 - R + rr, j.h, j.border);
        const uint32_t a = sbase + rr * 32 * 16;
        if (y < 0 || !live) {
          // A CONSTANT border row, or a lane no stored pixel reads.
          stage[rr * 32 + lane] = y < 0 ? make_uint4(bv4, bv4, bv4, bv4) : make_uint4(0u, 0u, 0u, 0u);
        } else {
          const uint8_t *row = j.src + static_cast<int64_t>(y) * j.src_stride;
          if (fast) {
            cp_async16g(a, row + 4 * e0);
          } else {
#pragma unroll
            for (int k = 0; k < kPix; ++k) {
              if (col[k] >= 0)
                cp_async4g(a + 4 * k, row + 4 * col[k]);
              else
                reinterpret_cast<uint32_t *>(stage + rr * 32 + lane)[k] = bv4;
            }
          }
        }
      }
      cp_async_commit_g();
    }
  }
  uint8_t *d = j.dst + static_cast<int64_t>(y0) * j.dst_stride + 4 * e0;
  // The byte-store path only where some lane of the warp needs it.
  if (__all_sync(0xffffffffu, !outputs || full_store))
    band_loop8<K, true>(j, stage, lane, rows, d, e0, outputs, full_store);
  else
    band_loop8<K, false>(j, stage, lane, rows, d, e0, outputs, full_store);
}

template <int K, bool SIMPLE>
__device__ __forceinline__ void band_loop8(const Gauss8Job &j, const uint4 *stage, int lane, int rows,
                                           uint8_t *d, long e0, bool outputs, bool full_store) {
  using G = GaussGeo<K>;
  constexpr int R = G::R;
  uint32_t wt[R + 1];
#pragma unroll
  for (int t = 0; t <= R; ++t) wt[t] = j.w8[t];
  // Window slot k holds the unpacked source row rr with rr = k mod K.
  uint32_t wl[K][kPix], wh[K][kPix];
  cp_async_wait_g<G::kGroups - 1>();  // group 0: rows 0 .. K - 1
#pragma unroll
  for (int rr = 0; rr < K - 1; ++rr) unpack4(stage[rr * 32 + lane], wl[rr], wh[rr]);
#pragma unroll 1
  for (int base = 0; base < rows; base += K) {
    // Destination rows base .. base + K - 1 read source rows up to
    // base + 2K - 2: groups up to base / K + 1.
    cp_async_wait_upto(max(0, G::kGroups - 2 - base / K));
    static_for<0, K>([&](auto sc) {
      constexpr int S = decltype(sc)::value;
      constexpr int slot = (S + K - 1) % K;  // receives source row base + S + K - 1
      if (base + S >= rows) return;  // past the band (the loop ends here)
      unpack4(stage[(base + S + K - 1) * 32 + lane], wl[slot], wh[slot]);
      const uint4 out = filter_row8<K, S>(wl, wh, wt);
      if (SIMPLE) {
        if (outputs) *reinterpret_cast<uint4 *>(d) = out;
      } else if (outputs) {
        if (full_store) {
          *reinterpret_cast<uint4 *>(d) = out;
        } else {
          const uint32_t o[4] = {out.x, out.y, out.z, out.w};
          const bool words = ((reinterpret_cast<uintptr_t>(j.dst) | static_cast<uintptr_t>(j.dst_stride)) & 3) == 0;
#pragma unroll
          for (int p = 0; p < kPix; ++p)
            if (e0 + p < j.w) {
              uint8_t *b = d + 4 * p;
              if (words) {
                *reinterpret_cast<uint32_t *>(b) = o[p];
              } else {  // any alignment: bytes
                b[0] = static_cast<uint8_t>(o[p]);
                b[1] = static_cast<uint8_t>(o[p] >> 8);
                b[2] = static_cast<uint8_t>(o[p] >> 16);
                b[3] = static_cast<uint8_t>(o[p] >> 24);
              }
            }
        }
      }
      d += j.dst_stride;
    });
  }
}

template <int K>
__global__ void __launch_bounds__(kThreadsG, K == 7 ? 4 : 5) gauss8_kernel(const __grid_constant__ Gauss8Job j) {
  extern __shared__ __align__(16) uint4 stage8[];
  launch_dependents();
  grid_dependency_wait();  // the source may be the previous call's output
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint4 *stage = stage8 + warp * (kWarpStage / 16);
  // Items go round the CTAs first, so that every SM gets the same number.
  const int gw = warp * gridDim.x + blockIdx.x;
  const int nw = gridDim.x * kWarpsG;
  const int items = j.strips * j.bands;
  for (int t = gw; t < items; t += nw) {
    // Strips rotate by 7 per band: a warp's items do not all land on the
    // costlier strips at the row's ends.
    const int band = t / j.strips, q = t - band * j.strips;
    const int strip = static_cast<int>((q + 7L * band) % j.strips);
    run_band8<K>(j, stage, strip, band, lane);
  }
}

// Batch plans: one launch over a table of jobs of the same K.  Warp item t
// belongs to the first entry whose item_end exceeds t; the item boundaries
// are cached in shared memory for that search (a table in global memory
// would make every search a chain of dependent loads).
constexpr int kG8SearchEntries = 512;

template <int K>
__global__ void __launch_bounds__(kThreadsG, K == 7 ? 4 : 5)
    gauss8_batch_kernel(const Gauss8Job *__restrict__ E, int n) {
  extern __shared__ __align__(16) uint4 stage8b[];
  __shared__ int ends[kG8SearchEntries];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint4 *stage = stage8b + warp * (kWarpStage / 16);
  const bool cached = n <= kG8SearchEntries;
  if (cached)
    for (int k = threadIdx.x; k < n; k += blockDim.x) ends[k] = E[k].item_end;
  __syncthreads();
  const int total = E[n - 1].item_end;
  const int gw = warp * gridDim.x + blockIdx.x;
  const int nw = gridDim.x * kWarpsG;
  for (int t = gw; t < total; t += nw) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
      const int mid = (lo + hi) / 2;
      if ((cached ? ends[mid] : E[mid].item_end) > t) hi = mid;
      else lo = mid + 1;
    }
    const Gauss8Job &j = E[lo];
    const int local = t - (lo > 0 ? (cached ? ends[lo - 1] : E[lo - 1].item_end) : 0);
    const int band = local / j.strips, q = local - band * j.strips;
    const int strip = static_cast<int>((q + 7L * band) % j.strips);
    run_band8<K>(j, stage, strip, band, lane);
  }
}

// Bands of at most kGauss8MaxBand rows, as many as give `slots` warps the
// same number of items (one wave of n items per warp).
void size_bands8(Gauss8Job &j, long slots) {
  j.strips = (j.w + kStripPix - 1) / kStripPix;
  const long min_bands = (j.h + kGauss8MaxBand - 1) / kGauss8MaxBand;
  const long per_warp = std::max(1L, (min_bands * j.strips + slots - 1) / slots);
  j.bands = static_cast<int32_t>(std::min<long>(j.h, std::max(min_bands, per_warp * slots / j.strips)));
  j.band_q = j.h / j.bands;
  j.band_r = j.h % j.bands;
}

template <int K>
cudaError_t launch8(Gauss8Job &j, int sm_count, cudaStream_t stream) {
  auto kern = gauss8_kernel<K>;
  int occ = 0;
  const cudaError_t err = resident_ctas_per_sm<gauss8_kernel<K>>(kThreadsG, kSmemG, &occ);
  if (err != cudaSuccess) return err;
  const long resident = static_cast<long>(occ) * std::max(sm_count, 1);
  const long slots = resident * kWarpsG;
  // Every resident warp gets the same number of items.
  size_bands8(j, slots);
  const long items = static_cast<long>(j.strips) * j.bands;
  const long grid = std::max(1L, std::min(resident, (items + kWarpsG - 1) / kWarpsG));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(static_cast<unsigned>(grid));
  cfg.blockDim = dim3(kThreadsG);
  cfg.dynamicSmemBytes = kSmemG;
  cfg.stream = stream;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, j);
}

}  // namespace

bool gauss8_eligible(const FilterJob &f) {
  if (f.mode != MODE_SIGMA || f.channels != 4 || (f.ksize != 3 && f.ksize != 5 && f.ksize != 7)) return false;
  // Whole pixels: 4-byte cp.async of every source pixel.
  if (((reinterpret_cast<uintptr_t>(f.src) | static_cast<uintptr_t>(f.src_stride)) & 3) != 0) return false;
  // Item indices in 32 bits.
  return static_cast<long>(f.height) * (f.width / kStripPix + 1) < (1L << 30);
}

template <int K>
int batch_warps8(int sm_count) {
  int occ = 0;
  if (resident_ctas_per_sm<gauss8_batch_kernel<K>>(kThreadsG, kSmemG, &occ) != cudaSuccess) return 0;
  return occ * std::max(sm_count, 1) * kWarpsG;
}

template <int K>
cudaError_t launch_batch8(const Gauss8Job *table, int n, long items, int sm_count, cudaStream_t stream) {
  const int warps = batch_warps8<K>(sm_count);
  if (warps == 0) return cudaErrorInvalidValue;
  const long grid = std::max(1L, std::min<long>(warps / kWarpsG, (items + kWarpsG - 1) / kWarpsG));
  gauss8_batch_kernel<K><<<static_cast<unsigned>(grid), kThreadsG, kSmemG, stream>>>(table, n);
  return cudaGetLastError();
}

void gauss8_job(const FilterJob &f, Gauss8Job &j) {
  j = Gauss8Job{};
  j.src = f.src;
  j.dst = f.dst;
  j.src_stride = f.src_stride;
  j.dst_stride = f.dst_stride;
  j.w = f.width;
  j.h = f.height;
  j.border = f.border;
  j.border_value = f.border_value;
  for (int t = 0; t < f.ksize; ++t) j.w8[t] = static_cast<uint32_t>(f.wy[t]);
}

int gauss8_batch_warps(int ksize, int sm_count) {
  switch (ksize) {
    case 3: return batch_warps8<3>(sm_count);
    case 5: return batch_warps8<5>(sm_count);
    case 7: return batch_warps8<7>(sm_count);
  }
  return 0;
}

void gauss8_size_for_share(Gauss8Job &j, int warps) { size_bands8(j, std::max(warps, 1)); }

cudaError_t launch_gauss8_batch(int ksize, const Gauss8Job *table, int n, long items, int sm_count,
                                cudaStream_t stream) {
  if (n <= 0 || items <= 0) return cudaSuccess;
  switch (ksize) {
    case 3: return launch_batch8<3>(table, n, items, sm_count, stream);
    case 5: return launch_batch8<5>(table, n, items, sm_count, stream);
    case 7: return launch_batch8<7>(table, n, items, sm_count, stream);
  }
  return cudaErrorInvalidValue;
}

cudaError_t launch_gauss8(const FilterJob &f, int sm_count, cudaStream_t stream) {
  Gauss8Job j{};
  j.src = f.src;
  j.dst = f.dst;
  j.src_stride = f.src_stride;
  j.dst_stride = f.dst_stride;
  j.w = f.width;
  j.h = f.height;
  j.border = f.border;
  j.border_value = f.border_value;
  for (int t = 0; t < f.ksize; ++t) j.w8[t] = static_cast<uint32_t>(f.wy[t]);
  switch (f.ksize) {
    case 3: return launch8<3>(j, sm_count, stream);
    case 5: return launch8<5>(j, sm_count, stream);
    case 7: return launch8<7>(j, sm_count, stream);
  }
  return cudaErrorInvalidValue;
}

}  // namespace kcv
