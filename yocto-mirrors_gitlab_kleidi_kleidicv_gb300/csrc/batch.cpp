// Batched execution: many independent requests of uneven sizes, channel
// counts and filter sizes run through persistent kernels that claim tiles
// from device-side work-lists.
//
// A plan validates every request exactly as the single call would
// (statuses[i] is that call's return value), prepares the fused jobs (tile
// shape, ring depth, tensor maps), groups their tiles by kernel instantiation
// (mode, size, channels), orders each group's tiles largest first, and
// uploads the job table and the work-lists in one device allocation.  A
// launch resets the work counters and starts one persistent kernel per group
// on forked streams, so the groups run concurrently; blur-and-downsample
// requests go to the pyramid kernel and four-channel generated 3x3 / 5x5 /
// 7x7 Gaussians to the streaming kernel of gauss8.cu (one launch per channel
// count or kernel size, over an entry table), and arbitrary-size Gaussians
// (two-pass kernel with a scratch image) and copies run on a branch of their
// own.  With use_graph the whole
// launch is captured once into a CUDA graph and replayed.
#include <string.h>

#include <algorithm>
#include <map>
#include <tuple>
#include <vector>

#include "host.h"

namespace kcv {
namespace {

constexpr int kBatchThreads = 128;  // every batched kernel runs 4-warp CTAs
#ifndef KCV_BATCH_TILE_ROWS
#define KCV_BATCH_TILE_ROWS 64
#endif
constexpr int kBatchTileRows = KCV_BATCH_TILE_ROWS;  // output rows per tile (whole blocks)
constexpr int kMaxBranches = 8;

struct Group {
  FilterJob rep;  // selects the kernel instantiation
  std::vector<BatchTile> tiles;
  std::vector<uint64_t> cost;
  size_t smem = 0;
  int tile_off = 0, ntiles = 0, grid = 0;
};

template <typename T>
void to_taps(const int32_t *in, T *out) {
  for (int i = 0; i < 5; ++i) out[i] = static_cast<T>(in[i]);
}

kleidicv_error_t prepare_request(const kleidicv_gpu_request_t &r, Prepared *p) {
  const bool ext = r.allow_extensions != 0;
  const int border = static_cast<int>(r.border_type);
  switch (r.op) {
    case KLEIDICV_GPU_OP_GAUSSIAN_BLUR_U8:
      return prepare_gaussian(static_cast<const uint8_t *>(r.src), r.src_stride,
                              static_cast<uint8_t *>(r.dst), r.dst_stride, r.width, r.height,
                              r.channels, r.kernel_width, r.kernel_height, r.sigma_x, r.sigma_y,
                              border, ext, r.border_value, p);
    case KLEIDICV_GPU_OP_SEPARABLE_FILTER_2D_U8: {
      uint8_t kx[5], ky[5];
      to_taps(r.kernel_x, kx);
      to_taps(r.kernel_y, ky);
      return prepare_separable(1, r.src, r.src_stride, r.dst, r.dst_stride, r.width, r.height,
                               r.channels, kx, r.kernel_width, ky, r.kernel_height, border, ext,
                               r.border_value, p);
    }
    case KLEIDICV_GPU_OP_SEPARABLE_FILTER_2D_U16: {
      uint16_t kx[5], ky[5];
      to_taps(r.kernel_x, kx);
      to_taps(r.kernel_y, ky);
      return prepare_separable(2, r.src, r.src_stride, r.dst, r.dst_stride, r.width, r.height,
                               r.channels, kx, r.kernel_width, ky, r.kernel_height, border, ext,
                               r.border_value, p);
    }
    case KLEIDICV_GPU_OP_SEPARABLE_FILTER_2D_S16: {
      if (!ext) return KLEIDICV_ERROR_NOT_IMPLEMENTED;  // extension only
      int16_t kx[5], ky[5];
      to_taps(r.kernel_x, kx);
      to_taps(r.kernel_y, ky);
      return prepare_separable(3, r.src, r.src_stride, r.dst, r.dst_stride, r.width, r.height,
                               r.channels, kx, r.kernel_width, ky, r.kernel_height, border, true,
                               r.border_value, p);
    }
    case KLEIDICV_GPU_OP_BLUR_AND_DOWNSAMPLE_U8:
      return prepare_blurdown(static_cast<const uint8_t *>(r.src), r.src_stride, r.width,
                              r.height, static_cast<uint8_t *>(r.dst), r.dst_stride, r.channels,
                              border, ext, r.border_value, p);
  }
  return KLEIDICV_ERROR_NOT_IMPLEMENTED;
}

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

}  // namespace
}  // namespace kcv

using namespace kcv;

struct kleidicv_gpu_batch_plan {
  kleidicv_gpu_context *ctx = nullptr;
  // Blur-and-downsample requests by channel count (index C - 1): host entries
  // while planning, then one single-phase pyramid launch over a device table.
  std::vector<kcv::PyrEntry> pyr[4];
  kcv::PyrEntry *d_pyr[4] = {nullptr, nullptr, nullptr, nullptr};
  // Four-channel generated Gaussians by kernel size (index (K - 3) / 2).
  std::vector<kcv::Gauss8Job> g8[3];
  kcv::Gauss8Job *d_g8[3] = {nullptr, nullptr, nullptr};
  uint8_t *dmem = nullptr;
  size_t dmem_bytes = 0;
  FilterJob *d_jobs = nullptr;
  BatchTile *d_tiles = nullptr;
  int *d_next = nullptr;
  std::vector<Group> groups;
  std::vector<FilterJob> jobs;
  std::vector<GenericJob> generic;
  std::vector<size_t> generic_off, generic_stride;
  std::vector<Prepared> copies;
  size_t tiles_total = 0;
  std::vector<cudaStream_t> branches;
  std::vector<cudaEvent_t> joins;
  cudaEvent_t fork = nullptr;
  cudaGraphExec_t exec = nullptr;
  uint64_t kernels_per_launch = 0;
};

namespace {

kleidicv_error_t enqueue(kleidicv_gpu_batch_plan *p, cudaStream_t s) {
  kleidicv_gpu_context *ctx = p->ctx;
  cudaError_t e = cudaSuccess;
  if (!p->groups.empty()) e = cudaMemsetAsync(p->d_next, 0, p->groups.size() * sizeof(int), s);
  if (e == cudaSuccess) e = cudaEventRecord(p->fork, s);
  const size_t nb = p->branches.size();
  std::vector<bool> used(nb, false);
  for (size_t b = 0; b < nb && e == cudaSuccess; ++b) e = cudaStreamWaitEvent(p->branches[b], p->fork, 0);
  // Groups round-robin over the branches; the last branch also takes the
  // generic jobs and copies.
  size_t lane = 0;  // next branch, round robin
  for (size_t g = 0; g < p->groups.size() && e == cudaSuccess; ++g, ++lane) {
    const Group &gr = p->groups[g];
    BatchLaunch bl{p->d_jobs, p->d_tiles + gr.tile_off, gr.ntiles, p->d_next + g, gr.smem, gr.grid};
    const size_t b = nb ? lane % nb : 0;
    used[b] = true;
    e = launch_fused_batch(gr.rep, bl, ctx->d_err, nb ? p->branches[b] : s);
  }
  for (int c = 0; c < 4 && e == cudaSuccess; ++c) {
    if (p->pyr[c].empty()) continue;
    PyrLaunch L{};
    L.entries = p->d_pyr[c];
    L.phase_begin[0] = 0;
    L.phase_begin[1] = static_cast<int32_t>(p->pyr[c].size());
    L.phases = 1;
    L.channels = c + 1;
    L.barrier = reinterpret_cast<unsigned *>(ctx->d_err + 1);
    L.err_flag = ctx->d_err;
    const size_t b = nb ? lane++ % nb : 0;
    used[b] = true;
    e = launch_pyramid(L, ctx->sm_count, nb ? p->branches[b] : s);
  }
  for (int k = 0; k < 3 && e == cudaSuccess; ++k) {
    if (p->g8[k].empty()) continue;
    const size_t b = nb ? lane++ % nb : 0;
    used[b] = true;
    e = launch_gauss8_batch(3 + 2 * k, p->d_g8[k], static_cast<int>(p->g8[k].size()), p->g8[k].back().item_end,
                            ctx->sm_count, nb ? p->branches[b] : s);
  }
  cudaStream_t tail = nb ? p->branches[nb - 1] : s;
  for (size_t i = 0; i < p->generic.size() && e == cudaSuccess; ++i) {
    e = launch_generic_gaussian(p->generic[i], p->dmem + p->generic_off[i], p->generic_stride[i], tail);
    if (nb) used[nb - 1] = true;
  }
  for (const Prepared &c : p->copies) {
    if (e != cudaSuccess) break;
    e = cudaMemcpy2DAsync(c.dst, c.dst_stride, c.src, c.src_stride, c.row_bytes, c.rows,
                          cudaMemcpyDeviceToDevice, tail);
    if (nb) used[nb - 1] = true;
  }
  for (size_t b = 0; b < nb && e == cudaSuccess; ++b) {
    e = cudaEventRecord(p->joins[b], p->branches[b]);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, p->joins[b], 0);
  }
  (void)used;
  return cuda_status(ctx, e);
}

}  // namespace

extern "C" {

kleidicv_error_t kleidicv_gpu_batch_plan_create(const kleidicv_gpu_request_t *requests,
                                                size_t count, kleidicv_error_t *statuses,
                                                kleidicv_gpu_batch_plan_t **plan_out,
                                                kleidicv_gpu_context_t *ctx) {
  if (!plan_out || (count && !requests)) return KLEIDICV_ERROR_NULL_POINTER;
  *plan_out = nullptr;
  kleidicv_error_t e = resolve_context(ctx);
  if (e != KLEIDICV_OK) return e;
  DeviceGuard guard(ctx->device);
  auto *p = new kleidicv_gpu_batch_plan();
  p->ctx = ctx;

  std::map<std::tuple<int, int, int, int>, size_t> group_of;
  long g8_items_bound[3] = {0, 0, 0};
  size_t generic_bytes = 0;
  for (size_t i = 0; i < count; ++i) {
    Prepared pr;
    const kleidicv_error_t st = prepare_request(requests[i], &pr);
    if (statuses) statuses[i] = st;
    if (st != KLEIDICV_OK) continue;
    switch (pr.kind) {
      case Prepared::NOTHING:
        break;
      case Prepared::COPY:
        p->copies.push_back(pr);
        break;
      case Prepared::GENERIC: {
        const GenericJob &g = pr.generic;
        const size_t stride = align_up(static_cast<size_t>(g.width) * g.channels, 16);
        p->generic.push_back(g);
        p->generic_stride.push_back(stride);
        p->generic_off.push_back(generic_bytes);  // relative; rebased below
        generic_bytes += align_up(stride * g.height, 256);
        break;
      }
      case Prepared::FUSED: {
        if (gauss8_eligible(pr.fused)) {
          // Item counts of a table stay in 32 bits: at most rows x strips items
          // per request (bands <= rows), a group takes requests up to 2^30.
          const int k = (pr.fused.ksize - 3) / 2;
          const long most = static_cast<long>(pr.fused.height) * (pr.fused.width / kGauss8Lanes / 4 + 1);
          if (g8_items_bound[k] + most < (1L << 30)) {
            g8_items_bound[k] += most;
            Gauss8Job g;
            gauss8_job(pr.fused, g);  // bands sized once the request count is known
            p->g8[k].push_back(g);
            break;
          }
        }
        if (pr.fused.mode == MODE_BLURDOWN) {
          const FilterJob &f = pr.fused;
          PyrEntry en;
          pyr_entry(en, f.src, f.src_stride, f.dst, f.dst_stride, f.width, f.height, f.channels, f.border,
                    f.border_value, 1);  // bands sized once the request count is known
          p->pyr[f.channels - 1].push_back(en);
          break;
        }
        FilterJob j = pr.fused;
        // The batched kernels run fixed 4-warp CTAs over 64-row tiles with the
        // default ring (the autotune table is measured for whole-image calls).
        TileShape t{kBatchThreads, 0, 4, 0};
        // Whole blocks of output rows; bands are counted in 16 bits.
        const int mb = block_out_rows(j.mode, j.ksize);
        const int rows_min = (j.out_height + 65534) / 65535;
        t.tile_rows = (std::max(kBatchTileRows, rows_min) + mb - 1) / mb * mb;
        apply_tile_shape(j, t);
        encode_tma(j);
        j.big_bands = 0;
        j.row_tiles = (j.out_height + j.tile_rows - 1) / j.tile_rows;
        const auto key = std::make_tuple(j.mode, j.ksize, j.channels, j.narrow);
        auto it = group_of.find(key);
        if (it == group_of.end()) {
          it = group_of.emplace(key, p->groups.size()).first;
          p->groups.emplace_back();
          p->groups.back().rep = j;
        }
        Group &gr = p->groups[it->second];
        const uint32_t jid = static_cast<uint32_t>(p->jobs.size());
        gr.smem = std::max(gr.smem, fused_smem_bytes(j));
        const int m = block_out_rows(j.mode, j.ksize);
        for (int band = 0; band < j.row_tiles; ++band) {
          const int rows = std::min(j.tile_rows, j.out_height - band * j.tile_rows);
          for (int strip = 0; strip < j.strips; ++strip) {
            gr.tiles.push_back(BatchTile{jid, static_cast<uint16_t>(strip), static_cast<uint16_t>(band)});
            gr.cost.push_back(static_cast<uint64_t>((rows + m - 1) / m * m + j.ksize - 1) *
                              static_cast<uint64_t>(j.strip_out_bytes));
          }
        }
        p->jobs.push_back(j);
        break;
      }
    }
  }

  // Largest tiles first within each group; device layout [jobs][tiles][counters][scratch].
  std::vector<BatchTile> all_tiles;
  for (Group &gr : p->groups) {
    std::vector<size_t> order(gr.tiles.size());
    for (size_t k = 0; k < order.size(); ++k) order[k] = k;
    std::stable_sort(order.begin(), order.end(),
                     [&](size_t a, size_t b) { return gr.cost[a] > gr.cost[b]; });
    gr.tile_off = static_cast<int>(all_tiles.size());
    gr.ntiles = static_cast<int>(order.size());
    for (size_t k : order) all_tiles.push_back(gr.tiles[k]);
    BatchLaunch bl{nullptr, nullptr, gr.ntiles, nullptr, gr.smem, 0};
    const int occ = std::max(1, fused_batch_blocks_per_sm(gr.rep, bl));
    gr.grid = std::max(1, std::min(gr.ntiles, occ * ctx->sm_count));
    gr.tiles.clear();
    gr.cost.clear();
  }
  p->tiles_total = all_tiles.size();
  // Blur-and-downsample entries: bands sized for each request's share of the
  // pyramid kernel's resident warps, items counted through the table.
  size_t npyr_groups = 0, pyr_bytes[4] = {0, 0, 0, 0};
  for (int c = 0; c < 4; ++c) {
    std::vector<PyrEntry> &v = p->pyr[c];
    if (v.empty()) continue;
    ++npyr_groups;
    const int share = std::max(1, pyramid_warps(c + 1, ctx->sm_count) / static_cast<int>(v.size()));
    int32_t items = 0;
    for (PyrEntry &en : v) {
      pyr_entry(en, en.src, en.src_stride, en.dst, en.dst_stride, en.w, en.h, c + 1, en.border, en.border_value,
                share);
      items += en.item_end;
      en.item_end = items;
    }
    pyr_bytes[c] = align_up(v.size() * sizeof(PyrEntry), 256);
  }
  // Four-channel Gaussians: bands sized for each request's share of the
  // streaming kernel's resident warps, items counted through the table.
  size_t ng8_groups = 0, g8_bytes[3] = {0, 0, 0};
  for (int k = 0; k < 3; ++k) {
    std::vector<Gauss8Job> &v = p->g8[k];
    if (v.empty()) continue;
    ++ng8_groups;
    const int share = std::max(1, gauss8_batch_warps(3 + 2 * k, ctx->sm_count) / static_cast<int>(v.size()));
    int32_t items = 0;
    for (Gauss8Job &g : v) {
      gauss8_size_for_share(g, share);
      items += g.strips * g.bands;
      g.item_end = items;
    }
    g8_bytes[k] = align_up(v.size() * sizeof(Gauss8Job), 256);
  }
  const size_t jobs_bytes = align_up(p->jobs.size() * sizeof(FilterJob), 256);
  const size_t tiles_bytes = align_up(all_tiles.size() * sizeof(BatchTile), 256);
  const size_t next_bytes = align_up(p->groups.size() * sizeof(int), 256);
  const size_t pyr_total = pyr_bytes[0] + pyr_bytes[1] + pyr_bytes[2] + pyr_bytes[3];
  const size_t g8_total = g8_bytes[0] + g8_bytes[1] + g8_bytes[2];
  p->dmem_bytes = jobs_bytes + tiles_bytes + next_bytes + generic_bytes + pyr_total + g8_total;
  if (p->dmem_bytes) {
    p->dmem = static_cast<uint8_t *>(ctx_alloc(ctx, p->dmem_bytes));
    if (!p->dmem) {
      delete p;
      return KLEIDICV_ERROR_ALLOCATION;
    }
  }
  p->d_jobs = reinterpret_cast<FilterJob *>(p->dmem);
  p->d_tiles = reinterpret_cast<BatchTile *>(p->dmem + jobs_bytes);
  p->d_next = reinterpret_cast<int *>(p->dmem + jobs_bytes + tiles_bytes);
  for (size_t &off : p->generic_off) off += jobs_bytes + tiles_bytes + next_bytes;
  {
    size_t off = jobs_bytes + tiles_bytes + next_bytes + generic_bytes;
    for (int c = 0; c < 4; ++c) {
      if (!pyr_bytes[c]) continue;
      p->d_pyr[c] = reinterpret_cast<PyrEntry *>(p->dmem + off);
      off += pyr_bytes[c];
    }
    for (int k = 0; k < 3; ++k) {
      if (!g8_bytes[k]) continue;
      p->d_g8[k] = reinterpret_cast<Gauss8Job *>(p->dmem + off);
      off += g8_bytes[k];
    }
  }
  // Through the pinned upload ring: no wait for the stream's earlier work.
  cudaError_t ce = upload_async(ctx, p->d_jobs, p->jobs.data(), p->jobs.size() * sizeof(FilterJob));
  if (ce == cudaSuccess)
    ce = upload_async(ctx, p->d_tiles, all_tiles.data(), all_tiles.size() * sizeof(BatchTile));
  for (int c = 0; c < 4 && ce == cudaSuccess; ++c)
    if (p->d_pyr[c]) ce = upload_async(ctx, p->d_pyr[c], p->pyr[c].data(), p->pyr[c].size() * sizeof(PyrEntry));
  for (int k = 0; k < 3 && ce == cudaSuccess; ++k)
    if (p->d_g8[k]) ce = upload_async(ctx, p->d_g8[k], p->g8[k].data(), p->g8[k].size() * sizeof(Gauss8Job));
  const size_t nbranch = std::min<size_t>(kMaxBranches, p->groups.size() + npyr_groups + ng8_groups +
                                          ((p->generic.empty() && p->copies.empty()) ? 0 : 1));
  if (ce == cudaSuccess) {
    // The context's branch streams and events, created once and shared.
    std::lock_guard<std::mutex> lock(ctx->branch_mutex);
    if (!ctx->fork_event) ce = cudaEventCreateWithFlags(&ctx->fork_event, cudaEventDisableTiming);
    while (ce == cudaSuccess && ctx->branches.size() < nbranch) {
      cudaStream_t st;
      cudaEvent_t ev;
      ce = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
      if (ce != cudaSuccess) break;
      ce = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
      if (ce != cudaSuccess) {
        cudaStreamDestroy(st);
        break;
      }
      ctx->branches.push_back(st);
      ctx->branch_events.push_back(ev);
    }
    if (ce == cudaSuccess) {
      p->fork = ctx->fork_event;
      p->branches.assign(ctx->branches.begin(), ctx->branches.begin() + nbranch);
      p->joins.assign(ctx->branch_events.begin(), ctx->branch_events.begin() + nbranch);
    }
  }
  p->kernels_per_launch = p->groups.size() + npyr_groups + ng8_groups + 2 * p->generic.size();
  if (ce != cudaSuccess) {
    kleidicv_gpu_batch_plan_destroy(p);
    return cuda_status(ctx, ce);
  }
  *plan_out = p;
  return KLEIDICV_OK;
}

kleidicv_error_t kleidicv_gpu_batch_plan_launch(kleidicv_gpu_batch_plan_t *plan, int use_graph,
                                                kleidicv_gpu_context_t *ctx) {
  if (!plan) return KLEIDICV_ERROR_NULL_POINTER;
  if (!ctx) ctx = plan->ctx;
  if (ctx != plan->ctx) return KLEIDICV_ERROR_CONTEXT_MISMATCH;
  DeviceGuard guard(ctx->device);
  if (!use_graph) {
    kleidicv_error_t e = enqueue(plan, ctx->stream);
    if (e == KLEIDICV_OK) ctx->launches += plan->kernels_per_launch;
    return e;
  }
  if (!plan->exec) {
    // Capture on a private stream so that work already queued on the
    // context's stream is not captured.
    cudaStream_t cs;
    cudaError_t ce = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    if (ce != cudaSuccess) return cuda_status(ctx, ce);
    cudaGraph_t graph = nullptr;
    ce = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    kleidicv_error_t e = KLEIDICV_OK;
    if (ce == cudaSuccess) {
      e = enqueue(plan, cs);
      ce = cudaStreamEndCapture(cs, &graph);
    }
    if (ce == cudaSuccess && e == KLEIDICV_OK) ce = cudaGraphInstantiate(&plan->exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    cudaStreamDestroy(cs);
    if (e != KLEIDICV_OK) return e;
    if (ce != cudaSuccess) return cuda_status(ctx, ce);
  }
  cudaError_t ce = cudaGraphLaunch(plan->exec, ctx->stream);
  if (ce == cudaSuccess) ctx->launches += plan->kernels_per_launch;
  return cuda_status(ctx, ce);
}

kleidicv_error_t kleidicv_gpu_batch_plan_destroy(kleidicv_gpu_batch_plan_t *plan) {
  if (!plan) return KLEIDICV_ERROR_NULL_POINTER;
  DeviceGuard guard(plan->ctx->device);
  // Stream-ordered release: launches already enqueued finish first.
  // The branch streams and events belong to the context.
  if (plan->exec) cudaGraphExecDestroy(plan->exec);
  if (plan->dmem) ctx_free(plan->ctx, plan->dmem, plan->dmem_bytes);
  delete plan;
  return KLEIDICV_OK;
}

size_t kleidicv_gpu_batch_plan_tile_count(const kleidicv_gpu_batch_plan_t *plan) {
  return plan ? plan->tiles_total : 0;
}

kleidicv_error_t kleidicv_gpu_batch_submit(const kleidicv_gpu_request_t *requests, size_t count,
                                           kleidicv_error_t *statuses,
                                           kleidicv_gpu_context_t *ctx) {
  kleidicv_gpu_batch_plan_t *plan = nullptr;
  kleidicv_error_t e = kleidicv_gpu_batch_plan_create(requests, count, statuses, &plan, ctx);
  if (e != KLEIDICV_OK) return e;
  e = kleidicv_gpu_batch_plan_launch(plan, 0, nullptr);
  kleidicv_gpu_batch_plan_destroy(plan);
  return e;
}

}  // extern "C"
