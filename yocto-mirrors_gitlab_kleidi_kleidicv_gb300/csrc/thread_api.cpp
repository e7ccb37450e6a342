// Threaded-API entries (include/kleidicv_gpu_thread.h): KleidiCV's
// kleidicv_thread_* contract -- host images, a caller-provided scheduler,
// synchronous return -- with the filter on the GPU and the scheduler's tasks
// doing the host side of the transfers, plus a persistent worker pool that
// implements the scheduler contract.
#include "../../include/kleidicv_gpu_thread.h"

#include <cuda_runtime.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

#include "host.h"

// ---------------------------------------------------------------------------
// Worker pool (kleidicv_thread_parallel).  Every `parallel` call wakes all
// workers; each takes task indices from a shared counter, and the call
// returns once every worker has finished with this call's job, so a job's
// callback is never run after its call returned.
struct kleidicv_gpu_thread_pool {
  struct Job {
    kleidicv_thread_callback cb = nullptr;
    void *data = nullptr;
    unsigned count = 0;
  };
  std::vector<std::thread> workers;
  std::mutex m, call;
  std::condition_variable wake, done;
  uint64_t generation = 0;
  size_t finished = 0;
  bool stop = false;
  Job job;
  std::atomic<unsigned> next{0};
  std::atomic<int> error{KLEIDICV_OK};

  void run(const Job &j) {
    for (unsigned i; (i = next.fetch_add(1)) < j.count;) {
      const kleidicv_error_t e = j.cb(i, i + 1, j.data);
      if (e != KLEIDICV_OK) {
        int expected = KLEIDICV_OK;
        error.compare_exchange_strong(expected, static_cast<int>(e));
      }
    }
  }
  void worker() {
    uint64_t seen = 0;
    for (;;) {
      Job j;
      {
        std::unique_lock<std::mutex> l(m);
        wake.wait(l, [&] { return stop || generation != seen; });
        if (stop) return;
        seen = generation;
        j = job;
      }
      run(j);
      std::lock_guard<std::mutex> l(m);
      if (++finished == workers.size()) done.notify_all();
    }
  }
};

namespace {

using kcv::Prepared;

bool device_accessible(const void *p, bool *pinned) {
  cudaPointerAttributes a;
  *pinned = false;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  *pinned = a.type == cudaMemoryTypeHost;
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// Grows the context's pinned staging to `bytes`.
bool pinned_staging(kleidicv_gpu_context_t *ctx, size_t bytes) {
  if (ctx->pinned_bytes >= bytes) return true;
  if (ctx->pinned) cudaFreeHost(ctx->pinned);
  ctx->pinned = nullptr;
  ctx->pinned_bytes = 0;
  if (cudaHostAlloc(&ctx->pinned, bytes, cudaHostAllocPortable) != cudaSuccess) {
    cudaGetLastError();
    ctx->pinned = nullptr;
    return false;
  }
  ctx->pinned_bytes = bytes;
  return true;
}

struct HostImage {
  const uint8_t *ptr;
  size_t stride, row_bytes, rows;
};

// One side (source or destination) of a threaded call.
struct Side {
  HostImage img;
  bool on_device = false;  // device or managed memory: used in place
  bool pinned = false;     // page-locked host memory: copied without packing
  uint8_t *dev = nullptr;  // device image (pitch `pitch`)
  uint8_t *stage = nullptr;  // pinned packing area (pitch `pitch`)
  size_t pitch = 0, dev_bytes = 0;
  unsigned rows_per_task = 1, tasks = 0;
};

void plan_tasks(Side &s) {
  // Stripes of about 2 MiB, at most 1024 of them.
  const size_t target = 2u << 20;
  size_t rpt = std::max<size_t>(1, target / std::max<size_t>(s.img.row_bytes, 1));
  rpt = std::max(rpt, (s.img.rows + 1023) / 1024);
  s.rows_per_task = static_cast<unsigned>(rpt);
  s.tasks = static_cast<unsigned>((s.img.rows + rpt - 1) / rpt);
}

struct Transfer {
  kleidicv_gpu_context_t *ctx;
  Side *side;
  std::vector<cudaEvent_t> *events;
};

kleidicv_error_t cuda_fail(kleidicv_gpu_context_t *ctx, cudaError_t e) {
  return kcv::cuda_status(ctx, e);
}

// Upload task t: pack its rows into pinned memory (pageable source) and
// enqueue their host-to-device copy.
kleidicv_error_t upload_task(unsigned begin, unsigned end, void *data) {
  const Transfer &x = *static_cast<Transfer *>(data);
  Side &s = *x.side;
  kcv::DeviceGuard guard(x.ctx->device);
  for (unsigned t = begin; t < end; ++t) {
    const size_t r0 = static_cast<size_t>(t) * s.rows_per_task;
    const size_t r1 = std::min(s.img.rows, r0 + s.rows_per_task);
    cudaError_t e;
    if (s.pinned) {
      e = cudaMemcpy2DAsync(s.dev + r0 * s.pitch, s.pitch, s.img.ptr + r0 * s.img.stride,
                            s.img.stride, s.img.row_bytes, r1 - r0, cudaMemcpyHostToDevice,
                            x.ctx->stream);
    } else {
      for (size_t r = r0; r < r1; ++r)
        memcpy(s.stage + r * s.pitch, s.img.ptr + r * s.img.stride, s.img.row_bytes);
      e = cudaMemcpyAsync(s.dev + r0 * s.pitch, s.stage + r0 * s.pitch, (r1 - r0) * s.pitch,
                          cudaMemcpyHostToDevice, x.ctx->stream);
    }
    if (e != cudaSuccess) return cuda_fail(x.ctx, e);
  }
  return KLEIDICV_OK;
}

// Download task t: wait for its stripe's copy, then unpack it into dst.
kleidicv_error_t download_task(unsigned begin, unsigned end, void *data) {
  const Transfer &x = *static_cast<Transfer *>(data);
  Side &s = *x.side;
  kcv::DeviceGuard guard(x.ctx->device);
  for (unsigned t = begin; t < end; ++t) {
    const cudaError_t e = cudaEventSynchronize((*x.events)[t]);
    if (e != cudaSuccess) return cuda_fail(x.ctx, e);
    const size_t r0 = static_cast<size_t>(t) * s.rows_per_task;
    const size_t r1 = std::min(s.img.rows, r0 + s.rows_per_task);
    uint8_t *dst = const_cast<uint8_t *>(s.img.ptr);
    for (size_t r = r0; r < r1; ++r)
      memcpy(dst + r * s.img.stride, s.stage + r * s.pitch, s.img.row_bytes);
  }
  return KLEIDICV_OK;
}

using DeviceOp = std::function<kleidicv_error_t(const void *, size_t, void *, size_t,
                                                kleidicv_gpu_context_t *)>;

// Pinned staging of asynchronous calls: buffers from the context's pool
// (reused), so that calls in flight never share staging.
void *pool_pinned(kleidicv_gpu_context_t *ctx, size_t bytes, size_t *got) {
  {
    std::lock_guard<std::mutex> l(ctx->pinned_pool_mutex);
    size_t best = ctx->pinned_pool.size();
    for (size_t i = 0; i < ctx->pinned_pool.size(); ++i)
      if (ctx->pinned_pool[i].second >= bytes &&
          (best == ctx->pinned_pool.size() || ctx->pinned_pool[i].second < ctx->pinned_pool[best].second))
        best = i;
    if (best < ctx->pinned_pool.size()) {
      auto b = ctx->pinned_pool[best];
      ctx->pinned_pool.erase(ctx->pinned_pool.begin() + best);
      *got = b.second;
      return b.first;
    }
  }
  void *p = nullptr;
  if (cudaHostAlloc(&p, bytes, cudaHostAllocPortable) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  *got = bytes;
  return p;
}

void pool_return(kleidicv_gpu_context_t *ctx, void *p, size_t bytes) {
  if (!p) return;
  std::lock_guard<std::mutex> l(ctx->pinned_pool_mutex);
  ctx->pinned_pool.emplace_back(p, bytes);
}

// One threaded call.  begin() validates the sides, runs the upload phase
// through the scheduler, enqueues the filter and the download copies (one
// copy and one event per destination stripe); complete() runs the download
// phase through the scheduler and releases the call's resources.  A
// synchronous call runs both on the caller's thread; an asynchronous one
// runs complete() on the context's completion worker.
struct ThreadedCall {
  kleidicv_gpu_context_t *ctx = nullptr;
  kleidicv_thread_multithreading mt{};
  bool async = false;
  Side s, d;
  std::vector<cudaEvent_t> events;
  cudaEvent_t done_event = nullptr;  // async: after the call's last copy
  void *staging = nullptr;           // async: pinned staging from the pool
  size_t staging_bytes = 0;

  kleidicv_error_t begin(const Prepared &p, HostImage src, HostImage dst, const DeviceOp &op);
  kleidicv_error_t complete(kleidicv_error_t result);
};

kleidicv_error_t ThreadedCall::begin(const Prepared &p, HostImage src, HostImage dst,
                                     const DeviceOp &op) {
  kcv::DeviceGuard guard(ctx->device);
  s.img = src;
  d.img = dst;
  // A single-row image may come with any stride (the reference ignores it).
  for (Side *x : {&s, &d})
    if (x->img.rows <= 1) x->img.stride = x->img.row_bytes;
  s.on_device = device_accessible(src.ptr, &s.pinned);
  d.on_device = device_accessible(dst.ptr, &d.pinned);
  auto pitch_of = [](size_t row_bytes) { return (row_bytes + 255) / 256 * 256; };
  for (Side *x : {&s, &d}) {
    if (x->on_device) {
      x->dev = const_cast<uint8_t *>(x->img.ptr);
      x->pitch = x->img.stride;
    } else {
      x->pitch = pitch_of(x->img.row_bytes);
      x->dev_bytes = x->pitch * x->img.rows;
      plan_tasks(*x);
    }
  }
  const size_t stage_s = (!s.on_device && !s.pinned) ? s.pitch * s.img.rows : 0;
  const size_t stage_d = (!d.on_device && !d.pinned) ? d.pitch * d.img.rows : 0;
  if (stage_s + stage_d > 0) {
    uint8_t *base;
    if (async) {
      staging = pool_pinned(ctx, stage_s + stage_d, &staging_bytes);
      if (!staging) return KLEIDICV_ERROR_ALLOCATION;
      base = static_cast<uint8_t *>(staging);
    } else {
      if (!pinned_staging(ctx, stage_s + stage_d)) return KLEIDICV_ERROR_ALLOCATION;
      base = static_cast<uint8_t *>(ctx->pinned);
    }
    s.stage = base;
    d.stage = base + stage_s;
  }
  if (s.dev_bytes) s.dev = static_cast<uint8_t *>(kcv::ctx_alloc(ctx, s.dev_bytes));
  if (d.dev_bytes) d.dev = static_cast<uint8_t *>(kcv::ctx_alloc(ctx, d.dev_bytes));
  if ((s.dev_bytes && !s.dev) || (d.dev_bytes && !d.dev)) return KLEIDICV_ERROR_ALLOCATION;

  // Upload phase: the scheduler runs the source stripes.
  kleidicv_error_t e;
  if (!s.on_device) {
    Transfer x{ctx, &s, nullptr};
    e = mt.parallel(upload_task, &x, mt.parallel_data, s.tasks);
    if (e != KLEIDICV_OK) return e;
  }
  e = op(s.dev, s.pitch, d.dev, d.pitch, ctx);
  if (e != KLEIDICV_OK) return e;
  if (!d.on_device) {
    events.resize(d.tasks, nullptr);
    for (unsigned t = 0; t < d.tasks; ++t) {
      const size_t r0 = static_cast<size_t>(t) * d.rows_per_task;
      const size_t r1 = std::min(d.img.rows, r0 + d.rows_per_task);
      cudaError_t ce = cudaEventCreateWithFlags(&events[t], cudaEventDisableTiming);
      if (ce == cudaSuccess) {
        if (d.pinned)
          ce = cudaMemcpy2DAsync(const_cast<uint8_t *>(d.img.ptr) + r0 * d.img.stride, d.img.stride,
                                 d.dev + r0 * d.pitch, d.pitch, d.img.row_bytes, r1 - r0,
                                 cudaMemcpyDeviceToHost, ctx->stream);
        else
          ce = cudaMemcpyAsync(d.stage + r0 * d.pitch, d.dev + r0 * d.pitch, (r1 - r0) * d.pitch,
                               cudaMemcpyDeviceToHost, ctx->stream);
      }
      if (ce == cudaSuccess) ce = cudaEventRecord(events[t], ctx->stream);
      if (ce != cudaSuccess) {
        events.resize(t + (events[t] ? 1 : 0));
        return cuda_fail(ctx, ce);
      }
    }
  }
  if (async) {
    cudaError_t ce = cudaEventCreateWithFlags(&done_event, cudaEventDisableTiming);
    if (ce == cudaSuccess) ce = cudaEventRecord(done_event, ctx->stream);
    if (ce != cudaSuccess) return cuda_fail(ctx, ce);
  }
  return KLEIDICV_OK;
}

kleidicv_error_t ThreadedCall::complete(kleidicv_error_t result) {
  kcv::DeviceGuard guard(ctx->device);
  // Download phase: the scheduler unpacks stripes as their copies land.
  if (result == KLEIDICV_OK && !d.on_device && !d.pinned && !events.empty()) {
    Transfer x{ctx, &d, &events};
    result = mt.parallel(download_task, &x, mt.parallel_data, d.tasks);
  }
  if (!s.on_device) kcv::ctx_free(ctx, s.dev, s.dev_bytes);
  if (!d.on_device) kcv::ctx_free(ctx, d.dev, d.dev_bytes);
  kleidicv_error_t se;
  if (async) {
    // Only this call's work: later calls on the stream need not have finished.
    const cudaError_t ce = done_event ? cudaEventSynchronize(done_event) : cudaSuccess;
    se = ce == cudaSuccess ? KLEIDICV_OK : cuda_fail(ctx, ce);
    if (done_event) cudaEventDestroy(done_event);
    done_event = nullptr;
    pool_return(ctx, staging, staging_bytes);
    staging = nullptr;
  } else {
    se = kleidicv_gpu_context_synchronize(ctx);
  }
  for (cudaEvent_t ev : events) cudaEventDestroy(ev);
  events.clear();
  return result != KLEIDICV_OK ? result : se;
}

kleidicv_error_t run_threaded(kleidicv_error_t validation, const Prepared &p, HostImage src,
                              HostImage dst, const DeviceOp &op,
                              kleidicv_thread_multithreading mt) {
  if (validation != KLEIDICV_OK) return validation;
  if (!mt.parallel) return KLEIDICV_ERROR_NULL_POINTER;
  if (p.kind == Prepared::NOTHING) return KLEIDICV_OK;
  ThreadedCall call;
  kleidicv_error_t e = kcv::resolve_context(call.ctx);
  if (e != KLEIDICV_OK) return e;
  call.mt = mt;
  e = call.begin(p, src, dst, op);
  return call.complete(e);
}

}  // namespace

// An asynchronous threaded call in flight (include/kleidicv_gpu_thread.h).
struct kleidicv_gpu_async {
  ThreadedCall call;
  kleidicv_gpu_async_callback done = nullptr;
  void *user_data = nullptr;
  bool caller_owns = false;
  mutable std::mutex m;
  std::condition_variable cv;
  bool complete = false;
  kleidicv_error_t status = KLEIDICV_OK;
};

namespace {

// Completion worker of a context: finishes queued asynchronous calls in
// submission order (they share the context's stream, so they also complete
// in that order).
void async_worker_loop(kleidicv_gpu_context_t *ctx) {
  for (;;) {
    kleidicv_gpu_async *a = nullptr;
    {
      std::unique_lock<std::mutex> l(ctx->async_mutex);
      ctx->async_cv.wait(l, [&] { return ctx->async_stop || !ctx->async_queue.empty(); });
      if (ctx->async_queue.empty()) return;  // stopping, nothing left
      a = ctx->async_queue.front();
      ctx->async_queue.pop_front();
    }
    const kleidicv_error_t st = a->call.complete(KLEIDICV_OK);
    if (a->done) a->done(st, a->user_data);
    if (!a->caller_owns) {
      delete a;
      continue;
    }
    // The caller may free the handle as soon as it sees `complete`: notify
    // under the lock and touch nothing afterwards.
    std::lock_guard<std::mutex> l(a->m);
    a->status = st;
    a->complete = true;
    a->cv.notify_all();
  }
}

kleidicv_error_t run_threaded_async(kleidicv_error_t validation, const Prepared &p, HostImage src,
                                    HostImage dst, const DeviceOp &op,
                                    kleidicv_thread_multithreading mt,
                                    kleidicv_gpu_async_callback done, void *user_data,
                                    kleidicv_gpu_async_t **handle) {
  if (handle) *handle = nullptr;
  if (validation != KLEIDICV_OK) return validation;
  if (!mt.parallel) return KLEIDICV_ERROR_NULL_POINTER;
  kleidicv_gpu_context_t *ctx = nullptr;
  kleidicv_error_t e = kcv::resolve_context(ctx);
  if (e != KLEIDICV_OK) return e;
  auto *a = new kleidicv_gpu_async();
  a->call.ctx = ctx;
  a->call.mt = mt;
  a->call.async = true;
  a->done = done;
  a->user_data = user_data;
  a->caller_owns = handle != nullptr;
  if (p.kind != Prepared::NOTHING) {
    e = a->call.begin(p, src, dst, op);
    if (e != KLEIDICV_OK) {
      a->call.complete(e);  // releases what begin() took
      delete a;
      return e;
    }
  }
  {
    std::lock_guard<std::mutex> l(ctx->async_mutex);
    if (!ctx->async_worker.joinable()) ctx->async_worker = std::thread(async_worker_loop, ctx);
    ctx->async_queue.push_back(a);
  }
  ctx->async_cv.notify_one();
  if (handle) *handle = a;
  return KLEIDICV_OK;
}

}  // namespace

extern "C" {

kleidicv_error_t kleidicv_gpu_thread_pool_create(kleidicv_gpu_thread_pool_t **pool,
                                                 unsigned threads) {
  if (!pool) return KLEIDICV_ERROR_NULL_POINTER;
  if (threads == 0) threads = std::max(1u, std::thread::hardware_concurrency());
  auto *p = new kleidicv_gpu_thread_pool();
  for (unsigned i = 1; i < threads; ++i) p->workers.emplace_back([p] { p->worker(); });
  *pool = p;
  return KLEIDICV_OK;
}

kleidicv_error_t kleidicv_gpu_thread_pool_destroy(kleidicv_gpu_thread_pool_t *pool) {
  if (!pool) return KLEIDICV_ERROR_NULL_POINTER;
  {
    std::lock_guard<std::mutex> l(pool->m);
    pool->stop = true;
  }
  pool->wake.notify_all();
  for (auto &t : pool->workers) t.join();
  delete pool;
  return KLEIDICV_OK;
}

kleidicv_error_t kleidicv_gpu_thread_pool_parallel(kleidicv_thread_callback callback,
                                                   void *callback_data, void *parallel_data,
                                                   unsigned task_count) {
  auto *p = static_cast<kleidicv_gpu_thread_pool *>(parallel_data);
  if (!p || !callback) return KLEIDICV_ERROR_NULL_POINTER;
  if (task_count == 0) return KLEIDICV_OK;
  std::lock_guard<std::mutex> one_call(p->call);
  kleidicv_gpu_thread_pool::Job j{callback, callback_data, task_count};
  {
    std::lock_guard<std::mutex> l(p->m);
    p->job = j;
    p->next = 0;
    p->error = KLEIDICV_OK;
    p->finished = 0;
    ++p->generation;
  }
  p->wake.notify_all();
  p->run(j);
  std::unique_lock<std::mutex> l(p->m);
  p->done.wait(l, [&] { return p->finished == p->workers.size(); });
  return static_cast<kleidicv_error_t>(p->error.load());
}

kleidicv_error_t kleidicv_gpu_thread_gaussian_blur_u8(
    const uint8_t *src, size_t src_stride, uint8_t *dst, size_t dst_stride, size_t width,
    size_t height, size_t channels, size_t kernel_width, size_t kernel_height, float sigma_x,
    float sigma_y, kleidicv_border_type_t border_type, kleidicv_thread_multithreading mt) {
  Prepared p;
  const kleidicv_error_t v =
      kcv::prepare_gaussian(src, src_stride, dst, dst_stride, width, height, channels,
                            kernel_width, kernel_height, sigma_x, sigma_y, border_type, false, 0,
                            &p);
  const size_t rb = width * channels;
  return run_threaded(
      v, p, {src, src_stride, rb, height}, {dst, dst_stride, rb, height},
      [&](const void *s, size_t ss, void *d, size_t ds, kleidicv_gpu_context_t *c) {
        return kleidicv_gpu_gaussian_blur_u8(static_cast<const uint8_t *>(s), ss,
                                             static_cast<uint8_t *>(d), ds, width, height, channels,
                                             kernel_width, kernel_height, sigma_x, sigma_y,
                                             border_type, c);
      },
      mt);
}

kleidicv_error_t kleidicv_gpu_thread_separable_filter_2d_u8(
    const uint8_t *src, size_t src_stride, uint8_t *dst, size_t dst_stride, size_t width,
    size_t height, size_t channels, const uint8_t *kernel_x, size_t kernel_width,
    const uint8_t *kernel_y, size_t kernel_height, kleidicv_border_type_t border_type,
    kleidicv_thread_multithreading mt) {
  Prepared p;
  const kleidicv_error_t v = kcv::prepare_separable(1, src, src_stride, dst, dst_stride, width,
                                                    height, channels, kernel_x, kernel_width,
                                                    kernel_y, kernel_height, border_type, false,
                                                    0, &p);
  const size_t rb = width * channels;
  return run_threaded(
      v, p, {src, src_stride, rb, height}, {dst, dst_stride, rb, height},
      [&](const void *s, size_t ss, void *d, size_t ds, kleidicv_gpu_context_t *c) {
        return kleidicv_gpu_separable_filter_2d_u8(static_cast<const uint8_t *>(s), ss,
                                                   static_cast<uint8_t *>(d), ds, width, height,
                                                   channels, kernel_x, kernel_width, kernel_y,
                                                   kernel_height, border_type, c);
      },
      mt);
}

kleidicv_error_t kleidicv_gpu_thread_separable_filter_2d_u16(
    const uint16_t *src, size_t src_stride, uint16_t *dst, size_t dst_stride, size_t width,
    size_t height, size_t channels, const uint16_t *kernel_x, size_t kernel_width,
    const uint16_t *kernel_y, size_t kernel_height, kleidicv_border_type_t border_type,
    kleidicv_thread_multithreading mt) {
  Prepared p;
  const kleidicv_error_t v = kcv::prepare_separable(2, src, src_stride, dst, dst_stride, width,
                                                    height, channels, kernel_x, kernel_width,
                                                    kernel_y, kernel_height, border_type, false,
                                                    0, &p);
  const size_t rb = width * channels * 2;
  return run_threaded(
      v, p, {reinterpret_cast<const uint8_t *>(src), src_stride, rb, height},
      {reinterpret_cast<const uint8_t *>(dst), dst_stride, rb, height},
      [&](const void *s, size_t ss, void *d, size_t ds, kleidicv_gpu_context_t *c) {
        return kleidicv_gpu_separable_filter_2d_u16(static_cast<const uint16_t *>(s), ss,
                                                    static_cast<uint16_t *>(d), ds, width, height,
                                                    channels, kernel_x, kernel_width, kernel_y,
                                                    kernel_height, border_type, c);
      },
      mt);
}

kleidicv_error_t kleidicv_gpu_thread_blur_and_downsample_u8(
    const uint8_t *src, size_t src_stride, size_t src_width, size_t src_height, uint8_t *dst,
    size_t dst_stride, size_t channels, kleidicv_border_type_t border_type,
    kleidicv_thread_multithreading mt) {
  Prepared p;
  const kleidicv_error_t v = kcv::prepare_blurdown(src, src_stride, src_width, src_height, dst,
                                                   dst_stride, channels, border_type, false, 0, &p);
  return run_threaded(
      v, p, {src, src_stride, src_width * channels, src_height},
      {dst, dst_stride, (src_width + 1) / 2 * channels, (src_height + 1) / 2},
      [&](const void *s, size_t ss, void *d, size_t ds, kleidicv_gpu_context_t *c) {
        return kleidicv_gpu_blur_and_downsample_u8(static_cast<const uint8_t *>(s), ss, src_width,
                                                   src_height, static_cast<uint8_t *>(d), ds,
                                                   channels, border_type, c);
      },
      mt);
}

static kleidicv_error_t thread_sobel(bool horizontal, const uint8_t *src, size_t src_stride,
                                     int16_t *dst, size_t dst_stride, size_t width,
                                     size_t height, size_t channels,
                                     kleidicv_thread_multithreading mt) {
  Prepared p;
  const kleidicv_error_t v = kcv::prepare_sobel(horizontal, src, src_stride, dst, dst_stride,
                                                width, height, channels, &p);
  return run_threaded(
      v, p, {src, src_stride, width * channels, height},
      {reinterpret_cast<const uint8_t *>(dst), dst_stride, 2 * width * channels, height},
      [&](const void *s, size_t ss, void *d, size_t ds, kleidicv_gpu_context_t *c) {
        const uint8_t *su = static_cast<const uint8_t *>(s);
        int16_t *di = static_cast<int16_t *>(d);
        return horizontal
                   ? kleidicv_gpu_sobel_3x3_horizontal_s16_u8(su, ss, di, ds, width, height,
                                                              channels, c)
                   : kleidicv_gpu_sobel_3x3_vertical_s16_u8(su, ss, di, ds, width, height,
                                                            channels, c);
      },
      mt);
}

}  // extern "C"

template <typename T>
static kleidicv_error_t thread_median(kcv::MedianElem elem, const T *src, size_t src_stride, T *dst,
                                      size_t dst_stride, size_t width, size_t height,
                                      size_t channels, size_t kernel_width, size_t kernel_height,
                                      kleidicv_border_type_t border_type,
                                      kleidicv_thread_multithreading mt,
                                      kleidicv_error_t (*entry)(const T *, size_t, T *, size_t, size_t,
                                                                size_t, size_t, size_t, size_t,
                                                                kleidicv_border_type_t,
                                                                kleidicv_gpu_context_t *)) {
  bool work = false;
  const kleidicv_error_t v =
      kcv::validate_median(elem, sizeof(T), src, src_stride, dst, dst_stride, width, height,
                           channels, kernel_width, kernel_height, border_type, &work);
  Prepared p;  // NOTHING unless the call has work
  if (work) p.kind = Prepared::FUSED;
  const size_t rb = width * channels * sizeof(T);
  return run_threaded(
      v, p, {reinterpret_cast<const uint8_t *>(src), src_stride, rb, height},
      {reinterpret_cast<const uint8_t *>(dst), dst_stride, rb, height},
      [&](const void *s, size_t ss, void *d, size_t ds, kleidicv_gpu_context_t *c) {
        return entry(static_cast<const T *>(s), ss, static_cast<T *>(d), ds, width, height, channels,
                     kernel_width, kernel_height, border_type, c);
      },
      mt);
}

extern "C" {

#define KCV_THREAD_MEDIAN(suffix, T, ELEM)                                                     \
  kleidicv_error_t kleidicv_gpu_thread_median_blur_##suffix(                                   \
      const T *src, size_t src_stride, T *dst, size_t dst_stride, size_t width, size_t height, \
      size_t channels, size_t kernel_width, size_t kernel_height,                              \
      kleidicv_border_type_t border_type, kleidicv_thread_multithreading mt) {                 \
    return thread_median<T>(kcv::ELEM, src, src_stride, dst, dst_stride, width, height,        \
                            channels, kernel_width, kernel_height, border_type, mt,            \
                            kleidicv_gpu_median_blur_##suffix);                                \
  }
KCV_THREAD_MEDIAN(s8, int8_t, MEDIAN_S8)
KCV_THREAD_MEDIAN(u8, uint8_t, MEDIAN_U8)
KCV_THREAD_MEDIAN(u16, uint16_t, MEDIAN_U16)
KCV_THREAD_MEDIAN(s16, int16_t, MEDIAN_S16)
KCV_THREAD_MEDIAN(u32, uint32_t, MEDIAN_U32)
KCV_THREAD_MEDIAN(s32, int32_t, MEDIAN_S32)
KCV_THREAD_MEDIAN(f32, float, MEDIAN_F32)
#undef KCV_THREAD_MEDIAN

kleidicv_error_t kleidicv_gpu_thread_sobel_3x3_horizontal_s16_u8(
    const uint8_t *src, size_t src_stride, int16_t *dst, size_t dst_stride, size_t width,
    size_t height, size_t channels, kleidicv_thread_multithreading mt) {
  return thread_sobel(true, src, src_stride, dst, dst_stride, width, height, channels, mt);
}

kleidicv_error_t kleidicv_gpu_thread_sobel_3x3_vertical_s16_u8(
    const uint8_t *src, size_t src_stride, int16_t *dst, size_t dst_stride, size_t width,
    size_t height, size_t channels, kleidicv_thread_multithreading mt) {
  return thread_sobel(false, src, src_stride, dst, dst_stride, width, height, channels, mt);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Asynchronous variants: the same validation and device work, finished by the
// context's completion worker.
extern "C" {

kleidicv_error_t kleidicv_gpu_thread_gaussian_blur_u8_async(
    const uint8_t *src, size_t src_stride, uint8_t *dst, size_t dst_stride, size_t width,
    size_t height, size_t channels, size_t kernel_width, size_t kernel_height, float sigma_x,
    float sigma_y, kleidicv_border_type_t border_type, kleidicv_thread_multithreading mt,
    kleidicv_gpu_async_callback done, void *user_data, kleidicv_gpu_async_t **handle) {
  Prepared p;
  const kleidicv_error_t v =
      kcv::prepare_gaussian(src, src_stride, dst, dst_stride, width, height, channels,
                            kernel_width, kernel_height, sigma_x, sigma_y, border_type, false, 0,
                            &p);
  const size_t rb = width * channels;
  return run_threaded_async(
      v, p, {src, src_stride, rb, height}, {dst, dst_stride, rb, height},
      [=](const void *s, size_t ss, void *d, size_t ds, kleidicv_gpu_context_t *c) {
        return kleidicv_gpu_gaussian_blur_u8(static_cast<const uint8_t *>(s), ss,
                                             static_cast<uint8_t *>(d), ds, width, height, channels,
                                             kernel_width, kernel_height, sigma_x, sigma_y,
                                             border_type, c);
      },
      mt, done, user_data, handle);
}

kleidicv_error_t kleidicv_gpu_thread_separable_filter_2d_u8_async(
    const uint8_t *src, size_t src_stride, uint8_t *dst, size_t dst_stride, size_t width,
    size_t height, size_t channels, const uint8_t *kernel_x, size_t kernel_width,
    const uint8_t *kernel_y, size_t kernel_height, kleidicv_border_type_t border_type,
    kleidicv_thread_multithreading mt, kleidicv_gpu_async_callback done, void *user_data,
    kleidicv_gpu_async_t **handle) {
  Prepared p;
  const kleidicv_error_t v = kcv::prepare_separable(1, src, src_stride, dst, dst_stride, width,
                                                    height, channels, kernel_x, kernel_width,
                                                    kernel_y, kernel_height, border_type, false,
                                                    0, &p);
  const size_t rb = width * channels;
  return run_threaded_async(
      v, p, {src, src_stride, rb, height}, {dst, dst_stride, rb, height},
      [=](const void *s, size_t ss, void *d, size_t ds, kleidicv_gpu_context_t *c) {
        return kleidicv_gpu_separable_filter_2d_u8(static_cast<const uint8_t *>(s), ss,
                                                   static_cast<uint8_t *>(d), ds, width, height,
                                                   channels, kernel_x, kernel_width, kernel_y,
                                                   kernel_height, border_type, c);
      },
      mt, done, user_data, handle);
}

kleidicv_error_t kleidicv_gpu_thread_separable_filter_2d_u16_async(
    const uint16_t *src, size_t src_stride, uint16_t *dst, size_t dst_stride, size_t width,
    size_t height, size_t channels, const uint16_t *kernel_x, size_t kernel_width,
    const uint16_t *kernel_y, size_t kernel_height, kleidicv_border_type_t border_type,
    kleidicv_thread_multithreading mt, kleidicv_gpu_async_callback done, void *user_data,
    kleidicv_gpu_async_t **handle) {
  Prepared p;
  const kleidicv_error_t v = kcv::prepare_separable(2, src, src_stride, dst, dst_stride, width,
                                                    height, channels, kernel_x, kernel_width,
                                                    kernel_y, kernel_height, border_type, false,
                                                    0, &p);
  const size_t rb = width * channels * 2;
  return run_threaded_async(
      v, p, {reinterpret_cast<const uint8_t *>(src), src_stride, rb, height},
      {reinterpret_cast<const uint8_t *>(dst), dst_stride, rb, height},
      [=](const void *s, size_t ss, void *d, size_t ds, kleidicv_gpu_context_t *c) {
        return kleidicv_gpu_separable_filter_2d_u16(static_cast<const uint16_t *>(s), ss,
                                                    static_cast<uint16_t *>(d), ds, width, height,
                                                    channels, kernel_x, kernel_width, kernel_y,
                                                    kernel_height, border_type, c);
      },
      mt, done, user_data, handle);
}

kleidicv_error_t kleidicv_gpu_thread_blur_and_downsample_u8_async(
    const uint8_t *src, size_t src_stride, size_t src_width, size_t src_height, uint8_t *dst,
    size_t dst_stride, size_t channels, kleidicv_border_type_t border_type,
    kleidicv_thread_multithreading mt, kleidicv_gpu_async_callback done, void *user_data,
    kleidicv_gpu_async_t **handle) {
  Prepared p;
  const kleidicv_error_t v = kcv::prepare_blurdown(src, src_stride, src_width, src_height, dst,
                                                   dst_stride, channels, border_type, false, 0, &p);
  return run_threaded_async(
      v, p, {src, src_stride, src_width * channels, src_height},
      {dst, dst_stride, (src_width + 1) / 2 * channels, (src_height + 1) / 2},
      [=](const void *s, size_t ss, void *d, size_t ds, kleidicv_gpu_context_t *c) {
        return kleidicv_gpu_blur_and_downsample_u8(static_cast<const uint8_t *>(s), ss, src_width,
                                                   src_height, static_cast<uint8_t *>(d), ds,
                                                   channels, border_type, c);
      },
      mt, done, user_data, handle);
}

kleidicv_error_t kleidicv_gpu_async_query(const kleidicv_gpu_async_t *handle) {
  if (!handle) return KLEIDICV_ERROR_NULL_POINTER;
  std::lock_guard<std::mutex> l(handle->m);
  return handle->complete ? handle->status : KLEIDICV_GPU_ERROR_NOT_READY;
}

kleidicv_error_t kleidicv_gpu_async_wait(kleidicv_gpu_async_t *handle) {
  if (!handle) return KLEIDICV_ERROR_NULL_POINTER;
  std::unique_lock<std::mutex> l(handle->m);
  handle->cv.wait(l, [&] { return handle->complete; });
  return handle->status;
}

kleidicv_error_t kleidicv_gpu_async_release(kleidicv_gpu_async_t *handle) {
  if (!handle) return KLEIDICV_ERROR_NULL_POINTER;
  kleidicv_gpu_async_wait(handle);
  delete handle;
  return KLEIDICV_OK;
}

}  // extern "C"

namespace kcv {

// Joins the context's completion worker after it has finished every queued
// call, and frees the pooled staging (kleidicv_gpu_context_destroy).
void shutdown_async(kleidicv_gpu_context_t *ctx) {
  {
    std::lock_guard<std::mutex> l(ctx->async_mutex);
    ctx->async_stop = true;
  }
  ctx->async_cv.notify_all();
  if (ctx->async_worker.joinable()) ctx->async_worker.join();
  std::lock_guard<std::mutex> l(ctx->pinned_pool_mutex);
  for (auto &b : ctx->pinned_pool) cudaFreeHost(b.first);
  ctx->pinned_pool.clear();
}

}  // namespace kcv
