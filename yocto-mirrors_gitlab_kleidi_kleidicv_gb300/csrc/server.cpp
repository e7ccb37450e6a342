// Serving loop: continuous batching of filter requests.
//
// Clients allocate request images from the server's device pool, submit
// requests at any time and poll completions.  A scheduler thread keeps up to
// max_inflight_batches batches on the GPU, each on its own stream: whenever
// a stream slot is free it admits the oldest queued requests (up to
// max_batch_requests, and only as many as the pool's free bytes cover for the
// batch's own device memory), builds a batch plan for them and launches it,
// while the batches already on the GPU keep running.  Finished batches are
// detected with events; their requests complete with the server-clock times
// of arrival, admission and completion.
#include <stdint.h>

#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "host.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Pending {
  uint64_t id;
  kleidicv_gpu_request_t req;
  double arrival_s;
};

struct Inflight {
  kleidicv_gpu_batch_plan_t *plan = nullptr;
  cudaEvent_t done = nullptr;
  std::vector<Pending> reqs;
  std::vector<kleidicv_error_t> statuses;
  double admitted_s = 0;
  size_t reserved = 0;
  int slot = 0;
};

// Device bytes a batch plan takes besides the request images: the job table,
// the work-lists and the two-pass scratch images (an upper bound).
size_t batch_bytes(const std::vector<Pending> &reqs) {
  size_t b = 4096;
  for (const Pending &p : reqs) {
    const kleidicv_gpu_request_t &r = p.req;
    b += sizeof(kcv::FilterJob) + 256;
    const size_t tiles = (r.width * r.channels * 2 / 1920 + 1) * (r.height / 32 + 1);
    b += tiles * sizeof(kcv::BatchTile);
    if (r.op == KLEIDICV_GPU_OP_GAUSSIAN_BLUR_U8 && r.kernel_width > 9 && r.kernel_width != 15 &&
        r.kernel_width != 21)
      b += (r.width * r.channels + 16) * r.height + 256;
  }
  return b;
}

}  // namespace

struct kleidicv_gpu_server {
  kleidicv_gpu_server_config_t cfg{};
  int device = 0;
  Clock::time_point t0;
  std::vector<kleidicv_gpu_context_t *> slots;  // one context (stream) per in-flight batch
  std::vector<bool> slot_busy;
  cudaStream_t alloc_stream = nullptr;
  cudaMemPool_t mempool = nullptr;
  size_t pool_used = 0;  // images + batch memory (guarded by mu)
  std::unordered_map<void *, size_t> allocations;

  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Pending> queue;
  std::vector<Inflight> inflight;
  std::deque<kleidicv_gpu_completion_t> completions;
  uint64_t next_id = 1;
  size_t outstanding = 0;
  bool stop = false;
  std::thread worker;

  double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }

  void retire_finished() {  // holds mu
    for (size_t i = 0; i < inflight.size();) {
      Inflight &f = inflight[i];
      const cudaError_t q = cudaEventQuery(f.done);
      if (q == cudaErrorNotReady) {
        ++i;
        continue;
      }
      kleidicv_error_t batch_status = KLEIDICV_OK;
      if (q != cudaSuccess) batch_status = KLEIDICV_GPU_ERROR_CUDA;
      else if (kleidicv_gpu_context_synchronize(slots[f.slot]) != KLEIDICV_OK)
        batch_status = KLEIDICV_GPU_ERROR_TIMEOUT;
      const double t = now();
      for (size_t k = 0; k < f.reqs.size(); ++k) {
        kleidicv_gpu_completion_t c;
        c.id = f.reqs[k].id;
        c.status = f.statuses[k] != KLEIDICV_OK ? f.statuses[k] : batch_status;
        c.arrival_s = f.reqs[k].arrival_s;
        c.admitted_s = f.admitted_s;
        c.completed_s = t;
        completions.push_back(c);
      }
      outstanding -= f.reqs.size();
      kleidicv_gpu_batch_plan_destroy(f.plan);
      cudaEventDestroy(f.done);
      pool_used -= f.reserved;
      slot_busy[f.slot] = false;
      inflight.erase(inflight.begin() + static_cast<long>(i));
      cv_done.notify_all();
    }
  }

  void run() {
    std::unique_lock<std::mutex> lock(mu);
    while (true) {
      retire_finished();
      if (stop && queue.empty() && inflight.empty()) break;
      // Admit into a free slot: oldest requests first, bounded by the batch
      // size and by the pool's free bytes.
      int slot = -1;
      for (size_t s = 0; s < slot_busy.size(); ++s)
        if (!slot_busy[s]) {
          slot = static_cast<int>(s);
          break;
        }
      if (slot >= 0 && !queue.empty()) {
        std::vector<Pending> batch;
        size_t need = 0;
        while (!queue.empty() && batch.size() < static_cast<size_t>(cfg.max_batch_requests)) {
          batch.push_back(queue.front());
          const size_t n = batch_bytes(batch);
          if (pool_used + n > cfg.pool_limit_bytes && batch.size() > 1) {
            batch.pop_back();
            break;
          }
          need = n;
          queue.pop_front();
        }
        if (pool_used + need > cfg.pool_limit_bytes && !inflight.empty()) {
          // Not even one request fits: wait for a batch to finish.
          for (auto it = batch.rbegin(); it != batch.rend(); ++it) queue.push_front(*it);
        } else {
          slot_busy[slot] = true;
          pool_used += need;
          const double admitted = now();
          lock.unlock();
          Inflight f;
          f.reqs = std::move(batch);
          f.slot = slot;
          f.reserved = need;
          f.admitted_s = admitted;
          std::vector<kleidicv_gpu_request_t> reqs(f.reqs.size());
          for (size_t k = 0; k < reqs.size(); ++k) reqs[k] = f.reqs[k].req;
          f.statuses.assign(reqs.size(), KLEIDICV_OK);
          kleidicv_error_t e = kleidicv_gpu_batch_plan_create(reqs.data(), reqs.size(),
                                                              f.statuses.data(), &f.plan, slots[slot]);
          if (e == KLEIDICV_OK) e = kleidicv_gpu_batch_plan_launch(f.plan, 0, slots[slot]);
          if (e == KLEIDICV_OK &&
              cudaEventCreateWithFlags(&f.done, cudaEventDisableTiming) != cudaSuccess)
            e = KLEIDICV_GPU_ERROR_CUDA;
          if (e == KLEIDICV_OK &&
              cudaEventRecord(f.done, kleidicv_gpu_context_get_stream_internal(slots[slot])) !=
                  cudaSuccess)
            e = KLEIDICV_GPU_ERROR_CUDA;
          lock.lock();
          if (e != KLEIDICV_OK) {
            // The whole batch fails with the plan's error.
            const double t = now();
            for (const Pending &p : f.reqs)
              completions.push_back({p.id, e, p.arrival_s, admitted, t});
            outstanding -= f.reqs.size();
            if (f.plan) kleidicv_gpu_batch_plan_destroy(f.plan);
            if (f.done) cudaEventDestroy(f.done);
            pool_used -= need;
            slot_busy[slot] = false;
            cv_done.notify_all();
          } else {
            inflight.push_back(std::move(f));
          }
          continue;
        }
      }
      // Nothing to admit: sleep until a submission, or poll the batches on
      // the GPU every 20 us.
      if (inflight.empty())
        cv_work.wait(lock, [&] { return stop || !queue.empty(); });
      else
        cv_work.wait_for(lock, std::chrono::microseconds(20));
    }
  }

  static cudaStream_t kleidicv_gpu_context_get_stream_internal(kleidicv_gpu_context_t *c) {
    return static_cast<cudaStream_t>(kleidicv_gpu_context_get_stream(c));
  }
};

extern "C" {

kleidicv_error_t kleidicv_gpu_server_create(const kleidicv_gpu_server_config_t *config, int device,
                                            kleidicv_gpu_server_t **out) {
  if (!out) return KLEIDICV_ERROR_NULL_POINTER;
  *out = nullptr;
  kleidicv_gpu_server_config_t cfg{};
  if (config) cfg = *config;
  if (!cfg.pool_limit_bytes) cfg.pool_limit_bytes = 40ull << 30;
  if (cfg.max_inflight_batches <= 0) cfg.max_inflight_batches = 4;
  if (cfg.max_batch_requests <= 0) cfg.max_batch_requests = 256;
  if (cfg.max_queue <= 0) cfg.max_queue = 65536;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) {
    cudaGetLastError();
    return KLEIDICV_GPU_ERROR_NO_DEVICE;
  }
  auto *s = new kleidicv_gpu_server();
  s->cfg = cfg;
  s->device = device;
  s->t0 = Clock::now();
  kcv::DeviceGuard guard(device);
  for (int i = 0; i < cfg.max_inflight_batches; ++i) {
    cudaStream_t st;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
      kleidicv_gpu_server_destroy(s);
      return KLEIDICV_GPU_ERROR_CUDA;
    }
    kleidicv_gpu_context_t *ctx = nullptr;
    // The server enforces the pool cap itself; each slot context may use it all.
    const kleidicv_error_t e = kleidicv_gpu_context_create(&ctx, device, st, cfg.pool_limit_bytes);
    if (e != KLEIDICV_OK) {
      cudaStreamDestroy(st);
      kleidicv_gpu_server_destroy(s);
      return e;
    }
    s->slots.push_back(ctx);
    s->slot_busy.push_back(false);
  }
  if (cudaStreamCreateWithFlags(&s->alloc_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaDeviceGetDefaultMemPool(&s->mempool, device) != cudaSuccess) {
    kleidicv_gpu_server_destroy(s);
    return KLEIDICV_GPU_ERROR_CUDA;
  }
  s->worker = std::thread([s] { s->run(); });
  *out = s;
  return KLEIDICV_OK;
}

kleidicv_error_t kleidicv_gpu_server_destroy(kleidicv_gpu_server_t *s) {
  if (!s) return KLEIDICV_ERROR_NULL_POINTER;
  if (s->worker.joinable()) {
    {
      std::lock_guard<std::mutex> lock(s->mu);
      s->stop = true;
    }
    s->cv_work.notify_all();
    s->worker.join();
  }
  kcv::DeviceGuard guard(s->device);
  for (auto &a : s->allocations) cudaFreeAsync(a.first, s->alloc_stream);
  if (s->alloc_stream) {
    cudaStreamSynchronize(s->alloc_stream);
    cudaStreamDestroy(s->alloc_stream);
  }
  for (kleidicv_gpu_context_t *c : s->slots) {
    cudaStream_t st = static_cast<cudaStream_t>(kleidicv_gpu_context_get_stream(c));
    kleidicv_gpu_context_destroy(c);
    cudaStreamDestroy(st);
  }
  delete s;
  return KLEIDICV_OK;
}

void *kleidicv_gpu_server_alloc(kleidicv_gpu_server_t *s, size_t bytes) {
  if (!s || !bytes) return nullptr;
  {
    std::lock_guard<std::mutex> lock(s->mu);
    if (s->pool_used + bytes > s->cfg.pool_limit_bytes) return nullptr;
    s->pool_used += bytes;
  }
  kcv::DeviceGuard guard(s->device);
  void *p = nullptr;
  if (cudaMallocFromPoolAsync(&p, bytes, s->mempool, s->alloc_stream) != cudaSuccess ||
      cudaStreamSynchronize(s->alloc_stream) != cudaSuccess) {
    std::lock_guard<std::mutex> lock(s->mu);
    s->pool_used -= bytes;
    return nullptr;
  }
  std::lock_guard<std::mutex> lock(s->mu);
  s->allocations[p] = bytes;
  return p;
}

void kleidicv_gpu_server_free(kleidicv_gpu_server_t *s, void *p) {
  if (!s || !p) return;
  size_t bytes = 0;
  {
    std::lock_guard<std::mutex> lock(s->mu);
    auto it = s->allocations.find(p);
    if (it == s->allocations.end()) return;
    bytes = it->second;
    s->allocations.erase(it);
  }
  kcv::DeviceGuard guard(s->device);
  cudaFreeAsync(p, s->alloc_stream);
  cudaStreamSynchronize(s->alloc_stream);
  std::lock_guard<std::mutex> lock(s->mu);
  s->pool_used -= bytes;
  s->cv_work.notify_all();
}

kleidicv_error_t kleidicv_gpu_server_submit(kleidicv_gpu_server_t *s,
                                            const kleidicv_gpu_request_t *request, uint64_t *id) {
  if (!s || !request) return KLEIDICV_ERROR_NULL_POINTER;
  {
    std::lock_guard<std::mutex> lock(s->mu);
    if (s->stop) return KLEIDICV_GPU_ERROR_BUSY;
    if (s->queue.size() >= static_cast<size_t>(s->cfg.max_queue)) return KLEIDICV_GPU_ERROR_BUSY;
    const uint64_t rid = s->next_id++;
    s->queue.push_back(Pending{rid, *request, s->now()});
    ++s->outstanding;
    if (id) *id = rid;
  }
  s->cv_work.notify_one();
  return KLEIDICV_OK;
}

size_t kleidicv_gpu_server_poll(kleidicv_gpu_server_t *s, kleidicv_gpu_completion_t *out,
                                size_t capacity, int timeout_ms) {
  if (!s || !out || !capacity) return 0;
  std::unique_lock<std::mutex> lock(s->mu);
  if (s->completions.empty() && timeout_ms > 0)
    s->cv_done.wait_for(lock, std::chrono::milliseconds(timeout_ms),
                        [&] { return !s->completions.empty(); });
  size_t n = 0;
  while (n < capacity && !s->completions.empty()) {
    out[n++] = s->completions.front();
    s->completions.pop_front();
  }
  return n;
}

double kleidicv_gpu_server_now(const kleidicv_gpu_server_t *s) { return s ? s->now() : 0.0; }

kleidicv_error_t kleidicv_gpu_server_drain(kleidicv_gpu_server_t *s) {
  if (!s) return KLEIDICV_ERROR_NULL_POINTER;
  std::unique_lock<std::mutex> lock(s->mu);
  s->cv_work.notify_all();
  s->cv_done.wait(lock, [&] { return s->outstanding == 0; });
  return KLEIDICV_OK;
}

}  // extern "C"
