// Serving loop: continuous batching of filter requests.
//
// Clients allocate request images from the server's device pool, submit
// requests at any time and poll completions.  Up to max_inflight_batches
// batches are on the GPU at once, one per slot (a worker thread with its own
// stream): a free worker admits the oldest queued requests (up to
// max_batch_requests and max_batch_bytes of image traffic, and only as many
// as the pool's free bytes cover for the batch's own device memory), builds a batch plan for them and launches it
// while the other slots' batches keep running.  Completion is detected with an
// event; its requests complete with the server-clock times of arrival,
// admission and completion.
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

// The request's image bytes read plus written: the unit of a batch's work
// budget (its GPU time is close to proportional to it).
size_t request_bytes(const kleidicv_gpu_request_t &r) {
  const size_t es =
      (r.op == KLEIDICV_GPU_OP_SEPARABLE_FILTER_2D_U16 || r.op == KLEIDICV_GPU_OP_SEPARABLE_FILTER_2D_S16) ? 2 : 1;
  const size_t in = r.width * r.height * r.channels * es;
  const size_t out = r.op == KLEIDICV_GPU_OP_BLUR_AND_DOWNSAMPLE_U8
                         ? ((r.width + 1) / 2) * ((r.height + 1) / 2) * r.channels
                         : in;
  return in + out;
}

}  // namespace

struct kleidicv_gpu_server {
  kleidicv_gpu_server_config_t cfg{};
  int device = 0;
  Clock::time_point t0;
  std::vector<kleidicv_gpu_context_t *> slots;  // one context (stream) per in-flight batch
  cudaStream_t alloc_stream = nullptr;
  cudaMemPool_t mempool = nullptr;
  size_t pool_used = 0;  // images + batch memory (guarded by mu)
  std::unordered_map<void *, size_t> allocations;

  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Pending> queue;
  std::deque<kleidicv_gpu_completion_t> completions;
  uint64_t next_id = 1;
  size_t outstanding = 0;
  int running = 0;  // batches on the GPU
  bool stop = false;
  std::vector<std::thread> workers;

  double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }

  // Takes the oldest queued requests that the pool's free bytes cover, up to
  // the batch work budget (at least one request) (holds mu).  Bounding a
  // batch's work bounds how long its requests, and the requests queued behind
  // it, wait for the GPU.
  std::vector<Pending> take_batch(size_t *need) {
    std::vector<Pending> batch;
    *need = 0;
    size_t work = 0;
    while (!queue.empty() && batch.size() < static_cast<size_t>(cfg.max_batch_requests)) {
      const size_t w = request_bytes(queue.front().req);
      if (!batch.empty() && work + w > cfg.max_batch_bytes) break;
      work += w;
      batch.push_back(queue.front());
      const size_t n = batch_bytes(batch);
      if (pool_used + n > cfg.pool_limit_bytes && batch.size() > 1) {
        batch.pop_back();
        break;
      }
      *need = n;
      queue.pop_front();
    }
    return batch;
  }

  // One worker per slot: take a batch, build and launch its plan on the
  // slot's stream, wait for it, publish the completions.  The workers build
  // plans concurrently, so a batch's preparation overlaps the other slots'
  // batches on the GPU.
  void work(int slot) {
    kleidicv_gpu_context_t *ctx = slots[slot];
    cudaStream_t stream = static_cast<cudaStream_t>(kleidicv_gpu_context_get_stream(ctx));
    cudaEvent_t done = nullptr;
    kcv::DeviceGuard guard(device);
    const cudaError_t ev_err = cudaEventCreateWithFlags(&done, cudaEventDisableTiming);
    std::unique_lock<std::mutex> lock(mu);
    while (true) {
      cv_work.wait(lock, [&] {
        return (stop && queue.empty()) ||
               (!queue.empty() && (running == 0 || pool_used + batch_bytes({queue.front()}) <=
                                                       cfg.pool_limit_bytes));
      });
      if (queue.empty()) break;  // stopping, nothing left
      size_t need = 0;
      std::vector<Pending> batch = take_batch(&need);
      pool_used += need;
      ++running;
      const double admitted = now();
      lock.unlock();

      std::vector<kleidicv_gpu_request_t> reqs(batch.size());
      for (size_t k = 0; k < reqs.size(); ++k) reqs[k] = batch[k].req;
      std::vector<kleidicv_error_t> statuses(reqs.size(), KLEIDICV_OK);
      kleidicv_gpu_batch_plan_t *plan = nullptr;
      kleidicv_error_t e = ev_err == cudaSuccess ? KLEIDICV_OK : KLEIDICV_GPU_ERROR_CUDA;
      if (e == KLEIDICV_OK)
        e = kleidicv_gpu_batch_plan_create(reqs.data(), reqs.size(), statuses.data(), &plan, ctx);
      if (e == KLEIDICV_OK) e = kleidicv_gpu_batch_plan_launch(plan, 0, ctx);
      if (e == KLEIDICV_OK && cudaEventRecord(done, stream) != cudaSuccess) e = KLEIDICV_GPU_ERROR_CUDA;
      if (e == KLEIDICV_OK) {
        // Poll (20 us) rather than block, so that the thread never holds the
        // device lock of a blocking synchronisation.
        cudaError_t q;
        while ((q = cudaEventQuery(done)) == cudaErrorNotReady)
          std::this_thread::sleep_for(std::chrono::microseconds(20));
        if (q != cudaSuccess) e = KLEIDICV_GPU_ERROR_CUDA;
        else if (kleidicv_gpu_context_synchronize(ctx) != KLEIDICV_OK) e = KLEIDICV_GPU_ERROR_TIMEOUT;
      }
      if (plan) kleidicv_gpu_batch_plan_destroy(plan);
      const double t = now();

      lock.lock();
      for (size_t k = 0; k < batch.size(); ++k) {
        kleidicv_gpu_completion_t c;
        c.id = batch[k].id;
        c.status = statuses[k] != KLEIDICV_OK ? statuses[k] : e;
        c.arrival_s = batch[k].arrival_s;
        c.admitted_s = admitted;
        c.completed_s = t;
        completions.push_back(c);
      }
      outstanding -= batch.size();
      pool_used -= need;
      --running;
      cv_done.notify_all();
      cv_work.notify_all();
    }
    lock.unlock();
    if (done) cudaEventDestroy(done);
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
  if (cfg.max_inflight_batches <= 0) cfg.max_inflight_batches = 3;
  if (cfg.max_batch_requests <= 0) cfg.max_batch_requests = 512;
  if (cfg.max_queue <= 0) cfg.max_queue = 65536;
  if (!cfg.max_batch_bytes) cfg.max_batch_bytes = ~static_cast<size_t>(0);
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
  }
  if (cudaStreamCreateWithFlags(&s->alloc_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaDeviceGetDefaultMemPool(&s->mempool, device) != cudaSuccess) {
    kleidicv_gpu_server_destroy(s);
    return KLEIDICV_GPU_ERROR_CUDA;
  }
  for (int i = 0; i < cfg.max_inflight_batches; ++i) s->workers.emplace_back([s, i] { s->work(i); });
  *out = s;
  return KLEIDICV_OK;
}

kleidicv_error_t kleidicv_gpu_server_destroy(kleidicv_gpu_server_t *s) {
  if (!s) return KLEIDICV_ERROR_NULL_POINTER;
  {
    std::lock_guard<std::mutex> lock(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  for (std::thread &t : s->workers)
    if (t.joinable()) t.join();
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
