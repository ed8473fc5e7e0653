// Serving loop: continuous batching of verification requests on one GPU.
//
// No counterpart in the reference (each call there builds a device and runs
// one batch, src/gpu.rs:5-35).  Requests (single- or mixed-curve batches of
// any size up to the slot capacity) are queued by sigops_server_submit; a
// dispatcher thread keeps K slots in flight, each with its own stream, pinned
// staging, device buffers and batched-engine scratch.  Whenever a slot is free
// and requests are waiting, it packs as many queued requests as fit into the
// slot and launches one batched step (H2D copy, classify, the fused kernel,
// D2H copy) on the slot's stream, so new arrivals join the next launch while
// earlier launches are still running and their kernels overlap on the device.
// Completed slots scatter results back to each request's output buffers.
//
// Admission: slot capacity and the queue bound come from free device memory
// at creation (cudaMemGetInfo x hbm_fraction); a request larger than a slot
// is refused with SIGOPS_E_RANGE and a submission that would push the queued
// items past the bound with SIGOPS_E_BUSY.
#include <cuda_runtime.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/sigops.h"
#include "launch.h"

namespace {

using Clock = std::chrono::steady_clock;

double now_s() { return std::chrono::duration<double>(Clock::now().time_since_epoch()).count(); }

struct Request {
  uint64_t id;
  const uint8_t *curves, *sigs, *msgs, *pks;
  int uniform_curve;  // >= 0 when `curves` is NULL
  size_t n;
  uint8_t *out, *status;
  double t_submit = 0, t_done = 0;
  int rc = SIGOPS_OK;
  bool done = false;
};

struct Slot {
  cudaStream_t stream = nullptr;
  sg::ForkStreams fork{};  // side streams: the single-curve variants run their three kernels side by side
  cudaEvent_t done = nullptr;
  uint8_t* h = nullptr;  // pinned staging: inputs then outputs
  uint8_t* d = nullptr;  // device buffer, same layout
  void* d_scratch = nullptr;
  uint32_t* d_idx = nullptr;
  void* d_defer = nullptr;  // shared-inversion scratch of the single-curve variants
  std::vector<Request*> reqs;
  size_t n = 0;
  bool busy = false;
};

struct Layout {
  size_t cur, sig, msg, pk, out, st, total;
};
Layout layout(size_t cap) {
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  Layout l;
  l.cur = 0;
  l.sig = al(cap);
  l.msg = l.sig + al(cap * 64);
  l.pk = l.msg + al(cap * 32);
  l.out = l.pk + al(cap * 32);
  l.st = l.out + al(cap * 64);
  l.total = l.st + al(cap);
  return l;
}

}  // namespace

struct sigops_server {
  sigops_ctx* ctx = nullptr;
  sg::CtxView cv{};
  std::vector<Slot> slots;
  size_t cap = 0;          // items per slot
  // batched-engine launch variant and its grid cap, packed in one word so the
  // worker reads a consistent pair (variant << 16 | blocks per launch at most).
  // Default: variant 1, the fused kernel with one tile per warp at 256 threads
  // (measured: the highest saturation).  The single-curve variants run their
  // three kernels side by side on the slot's side streams: lower latency at
  // light load, about 18% less saturation.  sigops_server_set_variant changes
  // it between launches.
  std::atomic<uint32_t> shape{0};
  size_t queue_bound = 0;  // max queued (not yet launched) items
  Layout lay{};
  std::mutex mu;
  std::condition_variable cond;
  std::deque<Request*> queue;
  size_t queued_items = 0;
  std::unordered_map<uint64_t, Request*> reqs;
  uint64_t next_id = 1;
  std::thread worker;
  bool stop = false;
  // stats
  uint64_t launches = 0, items_done = 0, requests_done = 0;
};

namespace {


// caller holds s->mu: move queued requests into the slot while they fit
void take_requests(sigops_server* s, Slot& sl) {
  sl.reqs.clear();
  size_t n = 0;
  while (!s->queue.empty() && n + s->queue.front()->n <= s->cap) {
    Request* r = s->queue.front();
    s->queue.pop_front();
    s->queued_items -= r->n;
    sl.reqs.push_back(r);
    n += r->n;
  }
  sl.n = n;
  sl.busy = n > 0;
}

// without the lock: pack the slot's requests into pinned staging and launch
void pack_and_launch(sigops_server* s, Slot& sl) {
  const size_t n = sl.n;
  const Layout& L = s->lay;
  size_t off = 0;
  for (Request* r : sl.reqs) {
    if (r->curves) memcpy(sl.h + L.cur + off, r->curves, r->n);
    else memset(sl.h + L.cur + off, r->uniform_curve, r->n);
    memcpy(sl.h + L.sig + off * 64, r->sigs, r->n * 64);
    memcpy(sl.h + L.msg + off * 32, r->msgs, r->n * 32);
    if (r->pks) memcpy(sl.h + L.pk + off * 32, r->pks, r->n * 32);
    else memset(sl.h + L.pk + off * 32, 0, r->n * 32);
    off += r->n;
  }
  cudaSetDevice(s->cv.device);
  // every call's status is kept: the first failure fails the slot's requests
  cudaError_t e = cudaSuccess;
  auto keep = [&e](cudaError_t r) {
    if (e == cudaSuccess) e = r;
  };
  keep(cudaMemcpyAsync(sl.d + L.cur, sl.h + L.cur, n, cudaMemcpyHostToDevice, sl.stream));
  keep(cudaMemcpyAsync(sl.d + L.sig, sl.h + L.sig, n * 64, cudaMemcpyHostToDevice, sl.stream));
  keep(cudaMemcpyAsync(sl.d + L.msg, sl.h + L.msg, n * 32, cudaMemcpyHostToDevice, sl.stream));
  keep(cudaMemcpyAsync(sl.d + L.pk, sl.h + L.pk, n * 32, cudaMemcpyHostToDevice, sl.stream));
  size_t cg = (n + 255) / 256;
  int classify_grid = (int)std::min(cg, (size_t)s->cv.num_sms * 8);
  // grid sized to the batch (the persistent variants: one item per thread up
  // to a full grid; the others size themselves): a light batch occupies few
  // SMs and launches from other slots run beside it
  const uint32_t shape = s->shape.load(std::memory_order_relaxed);
  const int variant = (int)(shape >> 16), grid_cap = (int)(shape & 0xffffu);
  const int block = sg::batched_variant_block(variant);
  const int grid = (int)std::min<size_t>((size_t)grid_cap, (n + block - 1) / block);
  keep(sg::launch_batched(sl.d + L.cur, sl.d + L.sig, sl.d + L.msg, sl.d + L.pk, n, sl.d + L.out, sl.d + L.st, sl.d_idx, sl.d_scratch,
                          sl.d_defer, s->cv.tabs, s->cv.d_err, grid, variant, classify_grid, &sl.fork, sl.stream));
  keep(cudaMemcpyAsync(sl.h + L.out, sl.d + L.out, n * 64, cudaMemcpyDeviceToHost, sl.stream));
  keep(cudaMemcpyAsync(sl.h + L.st, sl.d + L.st, n, cudaMemcpyDeviceToHost, sl.stream));
  keep(cudaEventRecord(sl.done, sl.stream));
  if (e != cudaSuccess) {
    for (Request* r : sl.reqs) r->rc = SIGOPS_E_CUDA;
  }
}

void finish(sigops_server* s, Slot& sl) {
  // caller holds s->mu
  const Layout& L = s->lay;
  cudaError_t e = cudaEventSynchronize(sl.done);
  double t = now_s();
  size_t off = 0;
  for (Request* r : sl.reqs) {
    if (e != cudaSuccess && r->rc == SIGOPS_OK) r->rc = SIGOPS_E_CUDA;
    memcpy(r->out, sl.h + L.out + off * 64, r->n * 64);
    if (r->status) memcpy(r->status, sl.h + L.st + off, r->n);
    off += r->n;
    r->t_done = t;
    r->done = true;
    s->requests_done++;
  }
  s->items_done += sl.n;
  sl.reqs.clear();
  sl.n = 0;
  sl.busy = false;
}

void worker_loop(sigops_server* s) {
  cudaSetDevice(s->cv.device);
  std::unique_lock<std::mutex> lk(s->mu);
  while (!s->stop) {
    bool progressed = false;
    for (Slot& sl : s->slots) {
      if (sl.busy && cudaEventQuery(sl.done) != cudaErrorNotReady) {
        finish(s, sl);
        progressed = true;
      }
    }
    if (progressed) s->cond.notify_all();
    for (Slot& sl : s->slots) {
      if (!sl.busy && !s->queue.empty()) {
        take_requests(s, sl);
        if (!sl.busy) continue;
        s->launches++;
        lk.unlock();
        pack_and_launch(s, sl);  // request buffers stay valid until completion
        lk.lock();
        progressed = true;
      }
    }
    if (!progressed) {
      bool any_busy = false;
      for (Slot& sl : s->slots) any_busy |= sl.busy;
      // poll completions every 20 us while work is in flight; otherwise sleep until a submit
      if (any_busy) s->cond.wait_for(lk, std::chrono::microseconds(20));
      else s->cond.wait_for(lk, std::chrono::milliseconds(5));
    }
  }
  for (Slot& sl : s->slots)
    if (sl.busy) finish(s, sl);
}

}  // namespace

extern "C" {

static int set_shape(sigops_server* s, int variant) {
  const int bps = sg::batched_max_blocks_per_sm(variant);
  if (bps <= 0) return SIGOPS_E_INVAL;
  const uint32_t grid_cap = std::min<uint32_t>(0xffffu, (uint32_t)(s->cv.num_sms * bps));
  s->shape.store(((uint32_t)variant << 16) | grid_cap, std::memory_order_relaxed);
  return SIGOPS_OK;
}

int sigops_server_set_variant(sigops_server* s, int variant) {
  if (!s || variant < 0 || variant >= sg::BATCHED_VARIANTS) return SIGOPS_E_INVAL;
  return set_shape(s, variant);
}

sigops_server* sigops_server_create(sigops_ctx* ctx, int nslots, size_t slot_items, double hbm_fraction) {
  sg::CtxView v;
  if (!ctx || sg::ctx_view(ctx, &v) != SIGOPS_OK) return nullptr;
  if (nslots <= 0) nslots = 8;
  if (nslots > 16) nslots = 16;
  if (hbm_fraction <= 0 || hbm_fraction > 0.9) hbm_fraction = 0.25;
  cudaSetDevice(v.device);
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return nullptr;
  const size_t per_item = 1 + 64 + 32 + 32 + 64 + 1 + 3 * 4;
  size_t budget_items = (size_t)(free_b * hbm_fraction) / per_item;
  if (slot_items == 0) slot_items = std::min<size_t>(budget_items / nslots, 1u << 14);
  if (slot_items == 0 || slot_items * nslots > budget_items) return nullptr;
  sigops_server* s = new sigops_server();
  s->ctx = ctx;
  s->cv = v;
  s->cap = slot_items;
  s->queue_bound = std::max<size_t>(slot_items * 64, budget_items);
  s->lay = layout(slot_items);
  if (set_shape(s, 1) != SIGOPS_OK) {
    delete s;
    return nullptr;
  }
  s->slots.resize(nslots);
  for (Slot& sl : s->slots) {
    bool ok = cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) == cudaSuccess &&
              sg::fork_streams_create(&sl.fork) == cudaSuccess &&
              cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming) == cudaSuccess &&
              cudaMallocHost(&sl.h, s->lay.total) == cudaSuccess && cudaMalloc(&sl.d, s->lay.total) == cudaSuccess &&
              cudaMalloc(&sl.d_scratch, sg::batched_scratch_bytes()) == cudaSuccess &&
              cudaMalloc(&sl.d_idx, 3 * slot_items * sizeof(uint32_t)) == cudaSuccess &&
              cudaMalloc(&sl.d_defer, sg::batched_defer_bytes(slot_items)) == cudaSuccess;
    if (!ok) {
      sigops_server_destroy(s);
      return nullptr;
    }
  }
  s->reqs.reserve(1u << 14);  // in-flight handles of a typical client without a rehash
  s->worker = std::thread(worker_loop, s);
  return s;
}

void sigops_server_destroy(sigops_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> g(s->mu);
    s->stop = true;
  }
  s->cond.notify_all();
  if (s->worker.joinable()) s->worker.join();
  cudaSetDevice(s->cv.device);
  for (Slot& sl : s->slots) {
    if (sl.stream) cudaStreamSynchronize(sl.stream);
    if (sl.done) cudaEventDestroy(sl.done);
    sg::fork_streams_destroy(&sl.fork);
    if (sl.stream) cudaStreamDestroy(sl.stream);
    if (sl.h) cudaFreeHost(sl.h);
    if (sl.d) cudaFree(sl.d);
    if (sl.d_scratch) cudaFree(sl.d_scratch);
    if (sl.d_idx) cudaFree(sl.d_idx);
    if (sl.d_defer) cudaFree(sl.d_defer);
  }
  for (auto& kv : s->reqs) delete kv.second;
  delete s;
}

size_t sigops_server_slot_items(sigops_server* s) { return s ? s->cap : 0; }

int sigops_server_submit(sigops_server* s, const uint8_t* curves, int uniform_curve, const uint8_t* sigs, const uint8_t* msgs,
                         const uint8_t* pks, size_t n, uint8_t* out, uint8_t* status, uint64_t* handle) {
  if (!s || !sigs || !msgs || !out || !handle || n == 0) return SIGOPS_E_INVAL;
  if (!curves && (uniform_curve < 0 || uniform_curve > 2)) return SIGOPS_E_INVAL;
  if (!curves && uniform_curve == SIGOPS_ED25519 && !pks) return SIGOPS_E_INVAL;
  if (n > s->cap) return SIGOPS_E_RANGE;
  Request* r = new Request();
  r->curves = curves;
  r->uniform_curve = curves ? -1 : uniform_curve;
  r->sigs = sigs;
  r->msgs = msgs;
  r->pks = pks;
  r->n = n;
  r->out = out;
  r->status = status;
  {
    std::lock_guard<std::mutex> g(s->mu);
    if (s->queued_items + n > s->queue_bound) {
      delete r;
      return SIGOPS_E_BUSY;
    }
    r->id = s->next_id++;
    r->t_submit = now_s();
    s->reqs[r->id] = r;
    s->queue.push_back(r);
    s->queued_items += n;
    *handle = r->id;
  }
  s->cond.notify_all();
  return SIGOPS_OK;
}

// Wait for a request; returns its result code (SIGOPS_OK), SIGOPS_E_TIMEDOUT
// if it is still running after timeout_ms (< 0: wait indefinitely), or
// SIGOPS_E_INVAL for an unknown handle.  A finished request is released.
int sigops_server_wait(sigops_server* s, uint64_t handle, int timeout_ms, double* latency_ms) {
  if (!s) return SIGOPS_E_INVAL;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->reqs.find(handle);
  if (it == s->reqs.end()) return SIGOPS_E_INVAL;
  Request* r = it->second;
  auto pred = [&] { return r->done; };
  if (timeout_ms < 0) s->cond.wait(lk, pred);
  else if (!s->cond.wait_for(lk, std::chrono::milliseconds(timeout_ms), pred)) return SIGOPS_E_TIMEDOUT;
  if (latency_ms) *latency_ms = (r->t_done - r->t_submit) * 1e3;
  int rc = r->rc;
  s->reqs.erase(it);
  delete r;
  return rc;
}

int sigops_server_stats(sigops_server* s, uint64_t* launches, uint64_t* requests_done, uint64_t* items_done, size_t* queued_items) {
  if (!s) return SIGOPS_E_INVAL;
  std::lock_guard<std::mutex> g(s->mu);
  if (launches) *launches = s->launches;
  if (requests_done) *requests_done = s->requests_done;
  if (items_done) *items_done = s->items_done;
  if (queued_items) *queued_items = s->queued_items;
  return SIGOPS_OK;
}

// Open-loop load: request i covers items [offset[i], offset[i] + count[i]) of
// the pool and is submitted at arrival_s[i] seconds after the start (arrivals
// in non-decreasing order); outputs land at the same item positions.  Fills
// latency_ms[i] (submit -> results in host memory) and the wall time from
// the first submission to the last completion.  Returns SIGOPS_E_BUSY if
// admission refused a request (its latency is set to -1).
int sigops_server_run_load(sigops_server* s, const uint8_t* curves, const uint8_t* sigs, const uint8_t* msgs, const uint8_t* pks,
                           const uint64_t* offset, const uint32_t* count, const double* arrival_s, size_t nreq, uint8_t* out,
                           uint8_t* status, double* latency_ms, double* wall_s) {
  if (!s || !curves || !sigs || !msgs || !pks || !offset || !count || !arrival_s || !out || !latency_ms) return SIGOPS_E_INVAL;
  std::vector<uint64_t> handles(nreq, 0);
  int rc = SIGOPS_OK;
  {
    // every request of the run is registered before the first wait: size the
    // handle table once, so that no rehash (which holds the server's lock for
    // milliseconds at a few hundred thousand entries) stalls the worker
    std::lock_guard<std::mutex> g(s->mu);
    s->reqs.reserve(s->reqs.size() + nreq);
  }
  const double t0 = now_s();
  for (size_t i = 0; i < nreq; ++i) {
    double target = t0 + arrival_s[i];
    for (;;) {
      double t = now_s();
      if (t >= target) break;
      if (target - t > 200e-6) std::this_thread::sleep_for(std::chrono::microseconds((int)((target - t - 100e-6) * 1e6)));
    }
    size_t o = offset[i];
    int r = sigops_server_submit(s, curves + o, -1, sigs + o * 64, msgs + o * 32, pks + o * 32, count[i], out + o * 64,
                                 status ? status + o : nullptr, &handles[i]);
    if (r != SIGOPS_OK) {
      handles[i] = 0;
      rc = r;
    }
  }
  for (size_t i = 0; i < nreq; ++i) {
    if (!handles[i]) {
      latency_ms[i] = -1;
      continue;
    }
    double lat = 0;
    int r = sigops_server_wait(s, handles[i], -1, &lat);
    latency_ms[i] = lat;
    if (r != SIGOPS_OK && rc == SIGOPS_OK) rc = r;
  }
  if (wall_s) *wall_s = now_s() - t0;
  return rc;
}

}  // extern "C"
