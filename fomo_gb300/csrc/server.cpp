// Render server: continuous batching of render requests as they arrive.
//
// Requests are submitted from any thread into a FIFO.  A scheduler thread
// owns the server's context and two launch slots, each with its own CUDA
// stream and scratch set.  Whenever a slot is free it admits every queued
// request that fits the HBM budget (output cube + descriptors) and the
// in-flight cap, plans them as one batch (one persistent march per launch
// group, shared neighbour lookups for requests with the same view) and
// enqueues it on the slot's stream.  While one slot's batch runs, requests
// that arrive meanwhile are admitted into the other slot, so their work
// overlaps on the device.  A slot's batch marches in view ranges of bounded
// work (a large view in launches of bounded work), launches with less work
// first and smaller images first within a launch; each range's cubes download
// as soon as it is done and its requests complete then, without waiting for the
// rest of the batch.  Each slot has a high- and a default-priority stream: a
// batch of small requests only goes on the high-priority one, so its kernels
// start ahead of a large request's next launch.  Results go
// device -> pinned staging -> the caller's buffer; each request records
// submit / admit / start / done times.
//
// A request is rendered by the same kernels, with the same per-ray work, as
// when it is rendered alone: one warp owns one ray and nothing in a ray's
// arithmetic depends on what else shares the launch.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/fomo_gpu.h"
#include "runtime_internal.h"

using namespace fomo;

namespace {

double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

enum class TState { kQueued, kRunning, kDone };

struct Ticket {
  fomo_request req{};
  float* out_host = nullptr;
  size_t out_bytes = 0;
  size_t cost = 0;  // admission bytes
  TState state = TState::kQueued;
  bool cancelled = false;
  int status = FOMO_OK;
  double t_submit = 0, t_admit = 0, t_start = 0, t_done = 0;
  size_t dev_off = 0, host_off = 0;
};

struct Slot {
  ScratchSet scr;
  cudaStream_t stream = nullptr;       // the stream of the batch in flight: one of the two below
  cudaStream_t stream_lo = nullptr;    // default priority: batches with a large request
  cudaStream_t stream_hi = nullptr;    // high priority: batches of small requests only
  cudaEvent_t done = nullptr;
  Arena out;              // device cubes of the batch
  char* pinned = nullptr; // host staging of the cubes
  size_t pinned_cap = 0;
  std::vector<uint64_t> ids;
  size_t cost = 0;        // admission bytes of the batch
  // view ranges of the batch in issue order: the event after each range's
  // downloads, and its requests
  std::vector<cudaEvent_t> evpool;
  std::deque<std::pair<cudaEvent_t, std::vector<uint64_t>>> ranges;
  bool busy = false;
  double t_launch = 0;
  // halting a batch whose requests were all cancelled: the march kernels
  // read halt_dev (ScratchSet::stop) before each ray; a cancellation sets it
  // with a copy on the server's control stream and records halt_ev after the
  // copy; the slot's next batch waits for halt_ev and clears the word first
  unsigned* halt_dev = nullptr;
  cudaEvent_t halt_ev = nullptr;
  bool halt_sent = false;
};

// Work per view range of a slot's batch (LOS samples + output cells): about a
// millisecond of march.  A larger view marches its rays in launches of about
// this much work too, so that the other slot's kernels can start in between.
constexpr double kServeRangeCost = double(1 << 24);
// A batch whose largest request has at most this many LOS samples goes on the
// slot's high-priority stream: its kernels are scheduled before a large
// request's as SMs free up.
constexpr double kServeSmallSamples = double(1 << 23);

}  // namespace

struct fomo_server {
  fomo_ctx* ctx = nullptr;
  std::thread worker;
  std::mutex mu;
  std::condition_variable cv;       // wakes the scheduler
  std::condition_variable done_cv;  // wakes waiters
  std::deque<uint64_t> queue;
  std::map<uint64_t, Ticket> tickets;
  uint64_t next_ticket = 1;
  size_t budget = 0;
  size_t inflight_bytes = 0;
  int max_inflight = 64;
  int inflight = 0;
  bool stop = false;
  Slot slots[2];
  cudaStream_t ctrl = nullptr;   // control copies (halt words), beside the slots' streams
  unsigned* halt_host = nullptr; // pinned {0, 1}: the halt word's two values
  std::string err;
  double t0 = 0;
};

namespace {

size_t request_cost(const fomo_request& q) {
  // output cube + per-view descriptors and tables (generous) + the deferred-sample and hard-sample queues
  const size_t rays = (size_t)(q.nx + 31) * (size_t)(q.ny + 31);  // tile padding included
  return cube_elems(q) * sizeof(float) + (size_t)q.nz * 24 + (size_t)(q.nx + q.ny) * 8 + 64 * 1024 +
         rays * (size_t)((q.nz + 63) / 64) * sizeof(DeferredRec) +
         (size_t)hard_capacity((int64_t)rays, q.nz) * sizeof(uint2) +
         (q.method != FOMO_METHOD_PROJECTION  // neighbour buffer and far-pass list
              ? rays * (size_t)q.nz * sizeof(int32_t) + rays * (size_t)((q.nz + 63) / 64) * sizeof(int32_t)
              : 0);
}

// Requests `ids` of slot sl are complete (their cubes are in pinned staging);
// called with S->mu held.
void finish_ids(fomo_server* S, Slot& sl, const std::vector<uint64_t>& ids, int status) {
  const double t = now_s() - S->t0;
  for (uint64_t id : ids) {
    auto it = S->tickets.find(id);
    if (it == S->tickets.end()) continue;
    Ticket& T = it->second;
    if (T.state == TState::kDone) continue;
    if (status == FOMO_OK && !T.cancelled && T.out_host)
      std::memcpy(T.out_host, sl.pinned + T.host_off, T.out_bytes);
    T.status = T.cancelled ? FOMO_ECANCELLED : status;
    T.state = TState::kDone;
    T.t_done = t;
  }
}

// The whole batch of slot sl is done: its remaining requests complete and its
// memory counts as free for admission; called with S->mu held.
void finish_slot(fomo_server* S, Slot& sl, int status) {
  finish_ids(S, sl, sl.ids, status);
  S->inflight_bytes -= sl.cost;
  S->inflight -= (int)sl.ids.size();
  sl.ids.clear();
  sl.ranges.clear();
  sl.cost = 0;
  sl.busy = false;
}

// Launch the admitted requests `ids` on slot `sl`; called without S->mu held.
int launch_slot(fomo_server* S, Slot& sl, std::vector<uint64_t>& ids, std::vector<fomo_request>& reqs,
                std::vector<size_t>& out_bytes) {
  NvtxRange range("fomo server: launch a batch");
  fomo_ctx* ctx = S->ctx;
  const int n = (int)reqs.size();
  std::vector<size_t> doff(n), hoff(n);
  size_t dtot = 0;
  for (int i = 0; i < n; ++i) {
    doff[i] = dtot;
    dtot += (out_bytes[i] + 255) & ~size_t(255);
  }
  int rc = sl.out.reserve(ctx, dtot);
  if (rc) return rc;
  if (sl.pinned_cap < dtot) {
    if (sl.pinned) cudaFreeHost(sl.pinned);
    sl.pinned = nullptr;
    sl.pinned_cap = 0;
    if (cudaMallocHost(reinterpret_cast<void**>(&sl.pinned), dtot) != cudaSuccess)
      return set_err(ctx, FOMO_ENOMEM, "pinned result staging");
    sl.pinned_cap = dtot;
  }
  std::vector<float*> d(n);
  for (int i = 0; i < n; ++i) d[i] = reinterpret_cast<float*>(sl.out.base + doff[i]);
  double largest = 0.0;
  for (const fomo_request& q : reqs) largest = std::max(largest, (double)q.nx * q.ny * q.nz);
  sl.stream = largest <= kServeSmallSamples ? sl.stream_hi : sl.stream_lo;
  cudaError_t eh = cudaStreamWaitEvent(sl.stream, sl.halt_ev, 0);
  if (eh == cudaSuccess)
    eh = cudaMemcpyAsync(sl.halt_dev, S->halt_host, sizeof(unsigned), cudaMemcpyHostToDevice, sl.stream);
  if (eh != cudaSuccess) return cuda_err(ctx, eh, "halt word");
  Plan plan;
  rc = plan_batch(ctx, reqs.data(), n, d.data(), nullptr, &sl.scr, &plan);
  if (rc) return rc;
  rc = order_streams(ctx, sl.stream);
  if (rc) return rc;
  // each view range: download its cubes, then an event that completes its requests
  std::deque<std::pair<cudaEvent_t, std::vector<uint64_t>>> ranges;
  size_t nev = 0;
  RangeDone done = [&](const PlanGroup& G, int v0, int v1) -> int {
    std::vector<uint64_t> rids;
    for (int v = v0; v < v1; ++v)
      for (int i : G.vreqs[v]) {
        cudaError_t e = cudaMemcpyAsync(sl.pinned + doff[i], d[i], out_bytes[i], cudaMemcpyDeviceToHost, sl.stream);
        if (e != cudaSuccess) return cuda_err(ctx, e, "result download");
        rids.push_back(ids[i]);
      }
    if (nev == sl.evpool.size()) {
      cudaEvent_t ev = nullptr;
      cudaError_t e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
      if (e != cudaSuccess) return cuda_err(ctx, e, "range event");
      sl.evpool.push_back(ev);
    }
    const cudaEvent_t ev = sl.evpool[nev++];
    cudaError_t e = cudaEventRecord(ev, sl.stream);
    if (e != cudaSuccess) return cuda_err(ctx, e, "range event");
    ranges.emplace_back(ev, std::move(rids));
    return FOMO_OK;
  };
  rc = issue_plan(ctx, plan, &sl.scr, sl.stream, &done, kServeRangeCost);
  if (rc) return rc;
  cudaError_t e = cudaEventRecord(sl.done, sl.stream);
  if (e != cudaSuccess) return cuda_err(ctx, e, "slot event");
  sl.ranges = std::move(ranges);  // only the scheduler thread (this one) reads them
  std::lock_guard<std::mutex> lk(S->mu);
  for (int i = 0; i < n; ++i) {
    auto it = S->tickets.find(ids[i]);
    if (it != S->tickets.end()) it->second.host_off = doff[i];
  }
  return FOMO_OK;
}

void scheduler(fomo_server* S) {
  cudaSetDevice(S->ctx->device);
  for (;;) {
    std::unique_lock<std::mutex> lk(S->mu);
    // completions: view ranges in issue order, then the whole batch
    for (Slot& sl : S->slots) {
      if (!sl.busy) continue;
      bool any = false;
      while (!sl.ranges.empty()) {
        const cudaError_t qr = cudaEventQuery(sl.ranges.front().first);
        if (qr == cudaErrorNotReady) break;
        if (qr != cudaSuccess) break;  // a device error: reported with the batch below
        finish_ids(S, sl, sl.ranges.front().second, FOMO_OK);
        sl.ranges.pop_front();
        any = true;
      }
      if (any) S->done_cv.notify_all();
      cudaError_t q = cudaEventQuery(sl.done);
      if (q == cudaSuccess) {
        finish_slot(S, sl, FOMO_OK);
        S->done_cv.notify_all();
      } else if (q != cudaErrorNotReady) {
        S->err = std::string("device error: ") + cudaGetErrorString(q);
        finish_slot(S, sl, FOMO_EDEVICE);
        S->done_cv.notify_all();
      }
    }
    const bool any_busy = S->slots[0].busy || S->slots[1].busy;
    if (S->stop && S->queue.empty() && !any_busy) break;
    // admission into a free slot
    Slot* free_slot = !S->slots[0].busy ? &S->slots[0] : (!S->slots[1].busy ? &S->slots[1] : nullptr);
    if (free_slot && !S->queue.empty()) {
      std::vector<uint64_t> ids;
      std::vector<fomo_request> reqs;
      std::vector<size_t> out_bytes;
      const double t = now_s() - S->t0;
      while (!S->queue.empty()) {
        uint64_t id = S->queue.front();
        Ticket& T = S->tickets[id];
        if (T.cancelled) {
          S->queue.pop_front();
          T.state = TState::kDone;
          T.status = FOMO_ECANCELLED;
          T.t_done = t;
          S->done_cv.notify_all();
          continue;
        }
        if (S->inflight > 0 && (S->inflight_bytes + T.cost > S->budget || S->inflight >= S->max_inflight)) break;
        S->queue.pop_front();
        T.state = TState::kRunning;
        T.t_admit = t;
        T.t_start = t;
        S->inflight_bytes += T.cost;
        S->inflight += 1;
        free_slot->cost += T.cost;
        ids.push_back(id);
        reqs.push_back(T.req);
        out_bytes.push_back(T.out_bytes);
      }
      if (!ids.empty()) {
        free_slot->busy = true;
        free_slot->ids = ids;
        free_slot->halt_sent = false;
        lk.unlock();
        int rc = launch_slot(S, *free_slot, ids, reqs, out_bytes);
        if (rc != FOMO_OK) cudaStreamSynchronize(free_slot->stream);  // part of the batch may be queued
        lk.lock();
        if (rc != FOMO_OK) {
          S->err = S->ctx->err;
          finish_slot(S, *free_slot, rc);
          S->done_cv.notify_all();
        }
        continue;
      }
    }
    // nothing to launch: wait for a submission or poll the device
    if (any_busy)
      S->cv.wait_for(lk, std::chrono::microseconds(100));
    else
      S->cv.wait_for(lk, std::chrono::milliseconds(50));
  }
}

}  // namespace

extern "C" {

int fomo_server_create(const fomo_server_config* config, fomo_server** out) {
  if (!config || !out) return FOMO_EINVAL;
  *out = nullptr;
  fomo_ctx* ctx = nullptr;
  int rc = fomo_ctx_create(config->device, 0, &ctx);
  if (rc) return rc;
  fomo_server* S = new fomo_server();
  S->ctx = ctx;
  size_t fr = 0, tot = 0;
  cudaMemGetInfo(&fr, &tot);
  S->budget = config->hbm_budget_bytes ? config->hbm_budget_bytes : fr / 2;
  S->max_inflight = config->max_inflight > 0 ? config->max_inflight : 64;
  for (Slot& sl : S->slots) {
    int lo = 0, hi = 0;
    cudaDeviceGetStreamPriorityRange(&lo, &hi);  // (least, greatest): greatest is numerically lowest
    if (sl.scr.init() != cudaSuccess ||
        cudaStreamCreateWithPriority(&sl.stream_lo, cudaStreamNonBlocking, lo) != cudaSuccess ||
        cudaStreamCreateWithPriority(&sl.stream_hi, cudaStreamNonBlocking, hi) != cudaSuccess ||
        cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming) != cudaSuccess) {
      fomo_ctx_destroy(ctx);
      delete S;
      return FOMO_EDEVICE;
    }
    sl.stream = sl.stream_lo;
  }
  bool ok = cudaStreamCreateWithFlags(&S->ctrl, cudaStreamNonBlocking) == cudaSuccess &&
            cudaMallocHost(reinterpret_cast<void**>(&S->halt_host), 2 * sizeof(unsigned)) == cudaSuccess;
  for (Slot& sl : S->slots)
    ok = ok && cudaMalloc(reinterpret_cast<void**>(&sl.halt_dev), 256) == cudaSuccess &&
         cudaMemset(sl.halt_dev, 0, sizeof(unsigned)) == cudaSuccess &&
         cudaEventCreateWithFlags(&sl.halt_ev, cudaEventDisableTiming) == cudaSuccess;
  if (!ok) {
    fomo_server_destroy(S);
    return FOMO_EDEVICE;
  }
  S->halt_host[0] = 0u;
  S->halt_host[1] = 1u;
  for (Slot& sl : S->slots) sl.scr.stop = sl.halt_dev;
  S->t0 = now_s();
  S->worker = std::thread(scheduler, S);
  *out = S;
  return FOMO_OK;
}

fomo_ctx* fomo_server_context(fomo_server* srv) { return srv ? srv->ctx : nullptr; }

int fomo_server_submit(fomo_server* S, const fomo_request* req, float* out_host, uint64_t* ticket) {
  if (!S || !req || !ticket) return FOMO_EINVAL;
  Ticket T;
  T.req = *req;
  T.out_host = out_host;
  T.out_bytes = cube_elems(*req) * sizeof(float);
  T.cost = request_cost(*req);
  std::lock_guard<std::mutex> lk(S->mu);
  if (req->nx < 2 || req->ny < 2 || req->nz < 1 || req->nlambda < 1) {
    S->err = "resolution must have nx >= 2, ny >= 2, nz >= 1, nlambda >= 1";
    return FOMO_EINVAL;
  }
  if (T.cost > S->budget) {
    S->err = "request needs " + std::to_string(T.cost) + " bytes, more than the server's HBM budget of " +
             std::to_string(S->budget);
    return FOMO_EADMISSION;
  }
  if (S->stop) {
    S->err = "server is stopping";
    return FOMO_ECANCELLED;
  }
  T.t_submit = now_s() - S->t0;
  const uint64_t id = S->next_ticket++;
  S->tickets[id] = T;
  S->queue.push_back(id);
  *ticket = id;
  S->cv.notify_all();
  return FOMO_OK;
}

int fomo_server_wait(fomo_server* S, uint64_t ticket, double timeout_s, fomo_request_stats* stats) {
  if (!S) return FOMO_EINVAL;
  std::unique_lock<std::mutex> lk(S->mu);
  auto it = S->tickets.find(ticket);
  if (it == S->tickets.end()) return FOMO_ENOTFOUND;
  const auto deadline = std::chrono::steady_clock::now() + std::chrono::duration<double>(timeout_s);
  while (S->tickets[ticket].state != TState::kDone) {
    if (S->done_cv.wait_until(lk, deadline) == std::cv_status::timeout &&
        S->tickets[ticket].state != TState::kDone)
      return FOMO_ETIMEOUT;
  }
  Ticket& T = S->tickets[ticket];
  if (stats) {
    stats->t_submit = T.t_submit;
    stats->t_admit = T.t_admit;
    stats->t_start = T.t_start;
    stats->t_done = T.t_done;
    stats->status = T.status;
  }
  const int st = T.status;
  S->tickets.erase(ticket);
  return st;
}

int fomo_server_cancel(fomo_server* S, uint64_t ticket) {
  if (!S) return FOMO_EINVAL;
  std::lock_guard<std::mutex> lk(S->mu);
  auto it = S->tickets.find(ticket);
  if (it == S->tickets.end()) return FOMO_ENOTFOUND;
  it->second.cancelled = true;  // queued: dropped at admission; running: result discarded
  if (it->second.state == TState::kRunning) {
    // a batch left with no request to deliver is halted on the device
    for (Slot& sl : S->slots) {
      if (!sl.busy || sl.halt_sent || std::find(sl.ids.begin(), sl.ids.end(), ticket) == sl.ids.end()) continue;
      bool all = true;
      for (uint64_t id : sl.ids) {
        auto jt = S->tickets.find(id);
        if (jt != S->tickets.end() && !jt->second.cancelled && jt->second.state != TState::kDone) all = false;
      }
      if (!all) continue;
      int prev = -1;
      cudaGetDevice(&prev);  // the caller's thread keeps its current device
      cudaSetDevice(S->ctx->device);
      if (cudaMemcpyAsync(sl.halt_dev, S->halt_host + 1, sizeof(unsigned), cudaMemcpyHostToDevice, S->ctrl) ==
              cudaSuccess &&
          cudaEventRecord(sl.halt_ev, S->ctrl) == cudaSuccess)
        sl.halt_sent = true;
      if (prev >= 0) cudaSetDevice(prev);
    }
  }
  S->cv.notify_all();
  return FOMO_OK;
}

int fomo_server_destroy(fomo_server* S) {
  if (!S) return FOMO_EINVAL;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
    S->cv.notify_all();
  }
  if (S->worker.joinable()) S->worker.join();
  for (Slot& sl : S->slots) {
    if (sl.stream_lo) cudaStreamSynchronize(sl.stream_lo);
    if (sl.stream_hi) cudaStreamSynchronize(sl.stream_hi);
    dev_free(S->ctx, sl.scr.arena.base);
    dev_free(S->ctx, sl.out.base);
    sl.scr.release();
    if (sl.pinned) cudaFreeHost(sl.pinned);
    for (cudaEvent_t ev : sl.evpool) cudaEventDestroy(ev);
    if (sl.done) cudaEventDestroy(sl.done);
    if (sl.stream_lo) cudaStreamDestroy(sl.stream_lo);
    if (sl.stream_hi) cudaStreamDestroy(sl.stream_hi);
    if (sl.halt_ev) cudaEventDestroy(sl.halt_ev);
    if (sl.halt_dev) cudaFree(sl.halt_dev);
  }
  if (S->ctrl) {
    cudaStreamSynchronize(S->ctrl);
    cudaStreamDestroy(S->ctrl);
  }
  if (S->halt_host) cudaFreeHost(S->halt_host);
  fomo_ctx_destroy(S->ctx);
  delete S;
  return FOMO_OK;
}

const char* fomo_server_last_error(fomo_server* S) { return S ? S->err.c_str() : "null server"; }

}  // extern "C"
