// The shard-proof server (apg_server_*, apg_submit, apg_poll, apg_wait in
// include/apogee_gpu.h): continuous batching of shard proofs on one GPU,
// built over the library's own C ABI.
//
// Requests queue in arrival order. The head of the queue is admitted when a
// worker is idle (or another can be added) and the bytes it may grow its
// worker's device holdings by fit the measured free HBM -- cudaMemGetInfo
// plus what the stream-ordered pool holds unused, minus the growth already
// reserved for running requests and the configured reserve -- and the
// budget. A worker is a context of its own (stream, scratch, second lane)
// sharing the owner's SRS, window tables and tuned widths, and a host thread
// that proves its request with apg_prove_shard; workers run side by side, so
// one request's host transcript steps and small launches overlap the others'
// kernels. A worker keeps its scratch between requests, so the next request
// routed to it grows nothing; routing prefers the idle worker that already
// holds the most.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/apogee_gpu.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
  uint64_t ticket = 0;
  apg_shard shard{};
  apg_shard_proof* out = nullptr;
  size_t need = 0;      // estimated peak device bytes of the request on an empty worker
  size_t reserved = 0;  // the growth reserved for it at admission
  int status = APG_PENDING;
  bool done = false;
  apg_request_times times{};
};

struct Worker {
  int id = 0;
  apg_ctx* ctx = nullptr;
  std::thread th;
  Request* job = nullptr;
  bool stop = false;
  size_t held = 0;  // device bytes its context held when it last went idle
  std::condition_variable cv;
};

// A context that has proved nothing yet still holds its flags and stream
// buffers; count a little for it.
constexpr size_t kWorkerBase = (size_t)64 << 20;
constexpr int kHardMaxWorkers = 64;

}  // namespace

struct apg_server {
  apg_ctx* owner = nullptr;
  int device = 0;
  apg_server_config cfg{};
  std::mutex mu;
  std::condition_variable done_cv;
  std::deque<Request*> queue;
  std::unordered_map<uint64_t, std::unique_ptr<Request>> reqs;
  std::vector<std::unique_ptr<Worker>> workers;
  uint64_t next_ticket = 1;
  uint64_t submitted = 0, completed = 0, failed = 0, in_flight = 0, peak_workers = 0, peak_in_flight = 0;
  size_t reserved = 0;
  double kernel_ms = 0, host_round_ms = 0;
  Clock::time_point t0 = Clock::now();

  uint64_t now_ns() const {
    return (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(Clock::now() - t0).count();
  }

  // Free device bytes as measured now: the driver's free count plus what the
  // stream-ordered pool holds and nobody uses. The caller's current device is
  // left as it was.
  size_t measured_free() const {
    int prev = device;
    cudaGetDevice(&prev);
    cudaSetDevice(device);
    size_t free_b = 0, total_b = 0;
    const bool ok = cudaMemGetInfo(&free_b, &total_b) == cudaSuccess;
    cudaSetDevice(prev);
    if (!ok) return 0;
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
      uint64_t res = 0, used = 0;
      if (cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &res) == cudaSuccess &&
          cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used) == cudaSuccess && res > used)
        free_b += (size_t)(res - used);
    }
    return free_b;
  }

  size_t held_total() const {
    size_t h = 0;
    for (auto& w : workers) h += w->held;
    return h;
  }

  Worker* spawn() {
    std::unique_ptr<Worker> w(new Worker());
    w->id = (int)workers.size();
    if (apg_ctx_create(device, &w->ctx) != APG_OK) return nullptr;
    if (apg_srs_share(w->ctx, owner) != APG_OK) {
      apg_ctx_destroy(w->ctx);
      return nullptr;
    }
    if (cfg.timing) apg_ctx_set_timing(w->ctx, 2);
    w->held = kWorkerBase;
    Worker* raw = w.get();
    raw->th = std::thread([this, raw] { run(raw); });
    workers.push_back(std::move(w));
    peak_workers = std::max<uint64_t>(peak_workers, workers.size());
    return raw;
  }

  // Admit from the head of the queue while a worker and the memory allow.
  // Called with `mu` held.
  void admit() {
    while (!queue.empty()) {
      Request* r = queue.front();
      Worker* w = nullptr;
      for (auto& x : workers)
        if (!x->job && !x->stop && (!w || x->held > w->held)) w = x.get();
      const size_t have = w ? w->held : 0;
      const size_t grow = r->need > have ? r->need - have : 0;
      const size_t extra = w ? 0 : kWorkerBase;
      const bool alone = in_flight == 0;
      if (!w && ((cfg.max_workers > 0 && (int)workers.size() >= cfg.max_workers) ||
                 (int)workers.size() >= kHardMaxWorkers))
        return;
      if (!alone) {  // the first request always runs: it either fits or fails with its own status
        if (measured_free() < reserved + grow + extra + cfg.hbm_reserve) return;
        if (cfg.hbm_budget && held_total() + reserved + grow + extra > cfg.hbm_budget) return;
      }
      if (!w) w = spawn();
      if (!w) {
        if (!alone) return;  // a running request will free a worker
        // Nothing runs and no worker can be made: the request fails rather
        // than waiting for memory that nothing will free.
        queue.pop_front();
        r->status = APG_ERR_OUT_OF_MEMORY;
        r->done = true;
        r->times.done_ns = now_ns();
        ++completed;
        ++failed;
        done_cv.notify_all();
        continue;
      }
      queue.pop_front();
      r->reserved = grow;
      reserved += grow;
      r->times.admit_ns = now_ns();
      r->times.reserved_bytes = grow;
      r->times.worker = w->id;
      ++in_flight;
      peak_in_flight = std::max(peak_in_flight, in_flight);
      w->job = r;
      w->cv.notify_one();
    }
  }

  void run(Worker* w) {
    std::unique_lock<std::mutex> lock(mu);
    for (;;) {
      w->cv.wait(lock, [w] { return w->job || w->stop; });
      if (!w->job) return;
      Request* r = w->job;
      r->times.start_ns = now_ns();
      lock.unlock();
      const int st = apg_prove_shard(w->ctx, &r->shard, r->out);
      const size_t held = apg_ctx_device_bytes(w->ctx) + kWorkerBase;
      double kms = 0, hms = 0;
      if (cfg.timing) {  // take the worker's totals and start it afresh
        uint64_t n = 0;
        apg_ctx_timer(w->ctx, APG_TIMER_KERNELS, &kms, &n);
        apg_ctx_timer(w->ctx, APG_TIMER_HOST_ROUND, &hms, &n);
        apg_ctx_set_timing(w->ctx, 2);
      }
      lock.lock();
      kernel_ms += kms;
      host_round_ms += hms;
      r->status = st;
      r->done = true;
      r->times.done_ns = now_ns();
      memcpy(r->times.phase_ms, r->out->phase_ms, sizeof(r->times.phase_ms));
      reserved -= r->reserved;
      w->held = held;
      w->job = nullptr;
      --in_flight;
      ++completed;
      if (st != APG_OK) ++failed;
      admit();
      done_cv.notify_all();
    }
  }
};

extern "C" {

int apg_server_create(apg_ctx* owner, const apg_server_config* cfg, apg_server** out) {
  if (!owner || !out) return APG_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  const int device = apg_ctx_device(owner);
  if (device < 0) return APG_ERR_NO_DEVICE;
  std::unique_ptr<apg_server> s(new apg_server());
  s->owner = owner;
  s->device = device;
  if (cfg) s->cfg = *cfg;
  *out = s.release();
  return APG_OK;
}

void apg_server_destroy(apg_server* s) {
  if (!s) return;
  {
    std::unique_lock<std::mutex> lock(s->mu);
    s->done_cv.wait(lock, [s] { return s->queue.empty() && s->in_flight == 0; });
    for (auto& w : s->workers) {
      w->stop = true;
      w->cv.notify_one();
    }
  }
  for (auto& w : s->workers) {
    if (w->th.joinable()) w->th.join();
    apg_ctx_destroy(w->ctx);
  }
  delete s;
}

int apg_submit(apg_server* s, const apg_shard* shard, apg_shard_proof* out, uint64_t* ticket) {
  if (!s || !shard || !out || !ticket) return APG_ERR_INVALID_ARGUMENT;
  std::unique_ptr<Request> r(new Request());
  r->shard = *shard;
  r->out = out;
  r->need = apg_shard_device_bytes(shard);
  if (r->need == 0) return APG_ERR_BAD_CIRCUIT;
  std::lock_guard<std::mutex> lock(s->mu);
  r->ticket = s->next_ticket++;
  r->times.submit_ns = s->now_ns();
  r->times.worker = -1;
  *ticket = r->ticket;
  s->queue.push_back(r.get());
  s->reqs[r->ticket] = std::move(r);
  ++s->submitted;
  s->admit();
  return APG_OK;
}

static int poll_locked(apg_server* s, uint64_t ticket, apg_request_times* times) {
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return APG_ERR_UNKNOWN_TICKET;
  Request* r = it->second.get();
  if (times) *times = r->times;
  return r->done ? r->status : APG_PENDING;
}

int apg_poll(apg_server* s, uint64_t ticket, apg_request_times* times) {
  if (!s) return APG_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(s->mu);
  return poll_locked(s, ticket, times);
}

int apg_wait(apg_server* s, uint64_t ticket, apg_request_times* times) {
  if (!s) return APG_ERR_INVALID_ARGUMENT;
  std::unique_lock<std::mutex> lock(s->mu);
  auto it = s->reqs.find(ticket);
  if (it == s->reqs.end()) return APG_ERR_UNKNOWN_TICKET;
  Request* r = it->second.get();
  s->done_cv.wait(lock, [r] { return r->done; });
  return poll_locked(s, ticket, times);
}

int apg_server_query(apg_server* s, apg_server_stats* out) {
  if (!s || !out) return APG_ERR_INVALID_ARGUMENT;
  std::lock_guard<std::mutex> lock(s->mu);
  out->submitted = s->submitted;
  out->completed = s->completed;
  out->failed = s->failed;
  out->queued = s->queue.size();
  out->in_flight = s->in_flight;
  out->workers = s->workers.size();
  out->peak_workers = s->peak_workers;
  out->peak_in_flight = s->peak_in_flight;
  out->held_bytes = s->held_total();
  out->reserved_bytes = s->reserved;
  out->kernel_ms = s->kernel_ms;
  out->host_round_ms = s->host_round_ms;
  return APG_OK;
}

}  // extern "C"
