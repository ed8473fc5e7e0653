// Serving loop: continuous batching of verification requests on one GPU.
//
// No counterpart in the reference (each call there builds a device and runs
// one batch, src/gpu.rs:5-35).  The queues live with the device:
//
//  * a pinned, mapped request ring on the host: sigops_server_submit copies a
//    request's items (signatures, messages, keys) into the item ring grouped
//    by curve, cuts them into 32-item single-curve tiles in the pinned tile
//    ring and publishes them (ServeCtl::tile_tail);
//  * one persistent kernel (serve.cuh, launched cooperatively so that all its
//    blocks are resident): a feeder warp copies published tiles into three
//    device-resident tile rings, one per curve, and every other warp claims
//    tiles of its TPC's current curve, copies their items from the pinned
//    rings into shared memory, verifies them and copies the results into the
//    pinned output ring; the warp whose tile completes a request appends it
//    to a pinned completion ring.
//
// Requests that arrive while others run become tiles behind them, and the
// warps of the one kernel take them up as they free: continuous batching with
// no launch, copy or host round trip per request.  The host reads the
// completion ring and copies each finished request's results to the caller's
// buffers: the dispatcher thread does, and so does every thread waiting for a
// request.  Both also relaunch the kernel when it has closed (idle, its
// lifetime cap, or a shape switch) and work is waiting, and fail the requests
// in flight if the kernel reports an expired device wait.  Apart from those
// launches no driver call is made while requests flow (the kernel reports its
// exit in a mapped word; free device memory is read by a monitor thread).
// With an adaptive shape (serve_policy.h) the dispatcher estimates the arrival
// rate and asks a launch of the other shape to close.
//
// Admission is live, at submit time: a request is admitted when the item ring
// (pinned; its tiles and counters in device memory, within hbm_fraction of
// the free device memory at creation), the tile rings and the request slots
// have room for it now, and while the device's free memory, re-read every
// 100 ms, stays above a floor (1% of the device, at least 256 MiB); else
// SIGOPS_E_BUSY.  A request larger than the per-request limit is refused with
// SIGOPS_E_RANGE.
#include <cuda_runtime.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/sigops.h"
#include "launch.h"
#include "serve.cuh"
#include "serve_policy.h"

namespace {

using Clock = std::chrono::steady_clock;

double now_s() { return std::chrono::duration<double>(Clock::now().time_since_epoch()).count(); }

enum class RState { Copying, Running, Finishing, Done, Canceled };

struct Request {
  uint64_t id = 0;
  uint32_t slot = 0, seq = 0;
  size_t off = 0, n = 0;
  uint64_t ring_end = 0;                  // item-ring position after this request (reclaimed in submission order)
  uint64_t tile_first = 0, tile_end = 0;  // its tiles in the tile rings
  uint8_t *out = nullptr, *status = nullptr;
  std::vector<uint32_t> perm;  // regrouped by curve: ring position -> the caller's item index (empty: same order)
  double t_submit = 0, t_done = 0;
  int rc = SIGOPS_OK;
  RState state = RState::Copying;
  bool ready = false;     // inputs copied, tiles written
  bool canceled = false;  // withdrawn by the caller: its results are dropped
};
using ReqPtr = std::shared_ptr<Request>;

// shapes of the persistent kernel (sigops_server_set_variant)
constexpr int kServeShapes = 3;
const int kServeBlock[kServeShapes] = {256, 128, 256};

}  // namespace

struct sigops_server {
  sigops_ctx* ctx = nullptr;
  sg::CtxView cv{};
  size_t max_items = 0;  // per request
  uint32_t C = 0;        // items in the rings
  uint32_t R = 0;        // request slots
  uint32_t tile_cap = 0;
  // pinned, mapped host memory
  sg::ServeCtl* ctl = nullptr;
  sg::ServeTile* htiles = nullptr;
  uint64_t* comp = nullptr;  // completion ring, R entries
  uint64_t comp_head = 0;    // entries consumed (dispatcher)
  uint8_t *sig = nullptr, *msg = nullptr, *pk = nullptr, *out = nullptr, *st = nullptr;
  void* host_block = nullptr;
  // device memory
  void* dev_block = nullptr;
  sg::ServeDev* dev = nullptr;
  sg::ServeTile* tiles = nullptr;
  uint32_t* count = nullptr;
  cudaStream_t stream = nullptr;
  cudaStream_t stat_stream = nullptr;  // reads of the kernel counters while it runs
  cudaEvent_t ev_exit = nullptr;
  bool running = false;
  uint32_t launch_no = 0;    // number of the running (or last) launch
  double exit_checked = 0;   // last driver-side look at the kernel (a fault would leave ServeCtl::exited unset)
  std::atomic<int> shape{0};
  // adaptive shape (sigops_server_set_adaptive; serve_policy.h); without it
  // every launch takes the fixed shape above
  sg::ShapePolicy policy;
  int running_shape = 0;    // shape of the running (or last) launch
  bool switching = false;   // the running launch was asked to close for a new shape
  double launched_at = 0;   // when it started
  uint64_t shape_switches = 0;
  uint64_t items_in = 0;    // items accepted by submit
  // host state, under mu
  std::mutex mu;
  std::condition_variable cond;
  std::unordered_map<uint64_t, ReqPtr> handles;
  std::vector<ReqPtr> by_slot;
  std::vector<uint32_t> slot_total;  // running item count of each request slot (the device's count)
  std::deque<ReqPtr> inflight;       // published, in submission order
  uint64_t next_id = 1;
  uint32_t next_seq = 1;
  uint64_t slots_taken = 0, published = 0;
  uint64_t item_head = 0, item_tail = 0;  // ring positions in use: [item_head, item_tail)
  uint64_t tile_head = 0, tile_alloc = 0, tiles_published = 0;
  size_t queued_items = 0;
  std::atomic<bool> hbm_ok{true};  // free device memory above the floor (monitor thread)
  size_t hbm_floor = 0;
  std::thread worker;
  std::thread monitor;  // re-reads free device memory every 100 ms (a driver call that can take milliseconds)
  bool stop = false;
  bool alive = true;    // the dispatcher runs
  bool broken = false;  // the kernel reported an expired wait, or could not launch: requests were failed
  int fault = 0;        // test hook: 1 = the dispatcher stops
  // stats
  uint64_t launches = 0, items_done = 0, requests_done = 0;
  uint64_t iterations = 0;
  double max_gap = 0;     // longest time between two dispatcher iterations since the last read (s)
  double max_driver = 0;  // longest driver call of the dispatcher since the last read (s)
};

namespace {

int grid_for(sigops_server* s, int shape, int* block) {
  int b = 0;
  cudaError_t e;
  *block = kServeBlock[shape];
  if (shape == 0) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, sg::serve_kernel<256, 1>, 256, 0);
  else if (shape == 1) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, sg::serve_kernel<128, 3>, 128, 0);
  else e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, sg::serve_kernel<256, 2>, 256, 0);
  return e == cudaSuccess ? b * s->cv.num_sms : 0;
}

// caller holds mu: the shape the next launch should have
int wanted_shape(const sigops_server* s) { return s->policy.wanted(s->shape.load(std::memory_order_relaxed), s->running_shape); }

// caller holds mu; the kernel is not running
cudaError_t launch_kernel(sigops_server* s) {
  const int shape = wanted_shape(s);
  s->running_shape = shape;
  s->switching = false;
  s->launched_at = now_s();
  __atomic_store_n(&s->ctl->stop, 0u, __ATOMIC_RELEASE);  // a shape switch's close request (destroy sets it only after the dispatcher ended)
  int block = 0;
  const int grid = grid_for(s, shape, &block);
  if (grid <= 0) return cudaErrorInvalidConfiguration;
  sg::ServeArgs a{};
  a.ctl = s->ctl;
  a.htiles = s->htiles;
  a.comp = s->comp;
  a.sig = s->sig;
  a.msg = s->msg;
  a.pk = s->pk;
  a.out = s->out;
  a.st = s->st;
  a.dev = s->dev;
  a.tiles = s->tiles;
  a.count = s->count;
  a.R = s->R;
  a.C = s->C;
  a.tile_cap = s->tile_cap;
  a.tabs = sg::BatchTables{s->cv.tabs.big[0], s->cv.tabs.big[1], s->cv.tabs.big[2], {nullptr, nullptr, nullptr}};
  a.idle_ns = 20ull * 1000 * 1000;    // close after 20 ms without a tile
  a.life_ns = 2000ull * 1000 * 1000;  // and after 2 s in all (the dispatcher relaunches)
  a.warps_per_sm = (uint32_t)(grid / s->cv.num_sms) * (uint32_t)(block / 32);
  a.warp_cap = 8 * sg::SERVE_SMS_PER_SLOT;  // 8 warps per SM: the 256 x 1 shape's full load
  a.launch = ++s->launch_no;
  sg::serve_reset_kernel<<<1, 1, 0, s->stream>>>(s->dev, (uint32_t)grid * (uint32_t)(block / 32));
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  void* args[] = {&a};
  if (shape == 0) e = cudaLaunchCooperativeKernel((const void*)sg::serve_kernel<256, 1>, grid, block, args, 0, s->stream);
  else if (shape == 1) e = cudaLaunchCooperativeKernel((const void*)sg::serve_kernel<128, 3>, grid, block, args, 0, s->stream);
  else e = cudaLaunchCooperativeKernel((const void*)sg::serve_kernel<256, 2>, grid, block, args, 0, s->stream);
  if (e != cudaSuccess) return e;
  return cudaEventRecord(s->ev_exit, s->stream);
}

// caller holds mu: every request in flight fails with rc (its results are not copied)
void fail_inflight(sigops_server* s, int rc) {
  const double t = now_s();
  for (ReqPtr& r : s->inflight) {
    if (r->state == RState::Running) {
      r->rc = rc;
      r->state = RState::Done;
      r->t_done = t;
    } else if (r->state == RState::Canceled) {
      r->state = RState::Done;
    }
  }
}

// caller holds mu: release finished requests at the front, in submission order
void reclaim(sigops_server* s) {
  while (!s->inflight.empty()) {
    ReqPtr& r = s->inflight.front();
    if (r->state != RState::Done) break;
    s->item_head = r->ring_end;
    s->tile_head = r->tile_end;
    s->queued_items -= r->n;
    s->by_slot[r->slot].reset();
    s->inflight.pop_front();
  }
}

// Completions: the kernel appends each finished request to the completion
// ring once its results are in the output ring.  The ring is read under the
// lock and the results are copied to the callers' buffers outside it.  The
// dispatcher calls this, and so does every thread waiting in
// sigops_server_wait: a dispatcher the OS leaves unscheduled for a few
// milliseconds then delays nothing.  Each caller copies its own disjoint set.
// Returns whether any request finished.
bool collect_completions(sigops_server* s, std::unique_lock<std::mutex>& lk, std::vector<ReqPtr>& finished) {
  finished.clear();
  bool changed = false;
  for (;;) {
    const uint64_t e = __atomic_load_n(&s->comp[s->comp_head % s->R], __ATOMIC_ACQUIRE);
    if ((uint32_t)e != (uint32_t)(s->comp_head + 1)) break;  // not written yet
    s->comp_head++;
    ReqPtr& r = s->by_slot[(e >> 32) & 0xffffu];
    if (!r || (r->seq & 0xffffu) != (uint32_t)(e >> 48)) continue;  // a request already failed on the host
    if (r->state == RState::Canceled) {
      r->state = RState::Done;  // results discarded
      changed = true;
    } else if (r->state == RState::Running) {
      r->state = RState::Finishing;
      finished.push_back(r);
    }
  }
  if (!finished.empty()) {
    lk.unlock();
    for (ReqPtr& r : finished) {
      if (r->perm.empty()) {
        memcpy(r->out, s->out + r->off * 64, r->n * 64);
        if (r->status) memcpy(r->status, s->st + r->off, r->n);
      } else {
        for (size_t p = 0; p < r->n; ++p) {
          memcpy(r->out + (size_t)r->perm[p] * 64, s->out + (r->off + p) * 64, 64);
          if (r->status) r->status[r->perm[p]] = s->st[r->off + p];
        }
      }
      r->t_done = now_s();
    }
    lk.lock();
    for (ReqPtr& r : finished) {
      r->state = RState::Done;
      s->requests_done++;
      s->items_done += r->n;
    }
    changed = true;
  }
  if (changed) {
    reclaim(s);
    s->cond.notify_all();
  }
  return changed;
}

// The persistent kernel, under the lock: notice its exit (its last warp writes
// ServeCtl::exited) and relaunch it when published tiles wait.  The
// dispatcher calls this, and so does every thread waiting in
// sigops_server_wait, so that a dispatcher the OS leaves unscheduled delays no
// relaunch.  driver_check: also ask the driver, every 50 ms, about a launch
// that has not reported its exit (a kernel that could not write the word);
// only the dispatcher does, since driver calls from other threads can hold a
// thread for milliseconds.  Returns whether requests failed.
bool service_kernel(sigops_server* s, bool driver_check) {
  bool changed = false;
  bool exited = false;
  if (s->running) {
    exited = __atomic_load_n(&s->ctl->exited, __ATOMIC_ACQUIRE) == s->launch_no;
    const double t = now_s();
    if (!exited && driver_check && t - s->exit_checked > 0.05) {
      s->exit_checked = t;
      exited = cudaEventQuery(s->ev_exit) != cudaErrorNotReady;
      s->max_driver = std::max(s->max_driver, now_s() - t);
    }
  }
  if (exited) {
    s->running = false;
    const uint32_t err = __atomic_exchange_n(&s->ctl->err, 0u, __ATOMIC_ACQ_REL);
    if (err) {
      // a device wait expired: tiles may be lost, so nothing in flight can be trusted
      s->broken = true;
      fail_inflight(s, SIGOPS_E_TIMEDOUT);
      changed = true;
    }
  }
  if (!s->running && !s->broken && !s->stop && __atomic_load_n(&s->ctl->tiles_fed, __ATOMIC_ACQUIRE) < s->tiles_published) {
    const double t = now_s();
    cudaError_t e = cudaSetDevice(s->cv.device);  // a waiting thread may not have the device current
    if (e == cudaSuccess) e = launch_kernel(s);
    s->max_driver = std::max(s->max_driver, now_s() - t);
    if (e == cudaSuccess) {
      s->running = true;
      s->launches++;
    } else {
      s->broken = true;
      fail_inflight(s, SIGOPS_E_CUDA);
      changed = true;
    }
  }
  return changed;
}

void worker_loop(sigops_server* s) {
  cudaSetDevice(s->cv.device);
  std::unique_lock<std::mutex> lk(s->mu);
  std::vector<ReqPtr> finished;
  double t_iter = now_s();
  bool busy = false;  // requests were in flight at the end of the previous iteration
  while (!s->stop) {
    if (s->fault == 1) break;  // test hook: the dispatcher stops as if it had died
    {
      const double t = now_s();
      if (busy) s->max_gap = std::max(s->max_gap, t - t_iter);
      t_iter = t;
      s->iterations++;
    }
    bool changed = collect_completions(s, lk, finished);
    {  // arrival rate; with an adaptive shape, a running launch of the other shape is asked to close
      const double t = now_s();
      s->policy.observe(t, s->items_in);
      if (s->running && !s->switching && s->policy.switch_rate > 0 && wanted_shape(s) != s->running_shape && t - s->launched_at > 0.02) {
        s->switching = true;
        s->shape_switches++;
        __atomic_store_n(&s->ctl->stop, 1u, __ATOMIC_RELEASE);  // the kernel finishes every published tile, then exits
      }
    }
    if (service_kernel(s, true)) changed = true;
    reclaim(s);
    if (changed) s->cond.notify_all();
    // poll completions every 20 us while requests are in flight
    busy = !s->inflight.empty();
    if (busy) s->cond.wait_for(lk, std::chrono::microseconds(20));
    else s->cond.wait_for(lk, std::chrono::milliseconds(5));
  }
  s->alive = false;
  s->cond.notify_all();
}

// admission by device memory: free memory re-read every 100 ms, on a thread
// of its own (the dispatcher makes no driver call while requests flow)
void monitor_loop(sigops_server* s) {
  cudaSetDevice(s->cv.device);
  std::unique_lock<std::mutex> lk(s->mu);
  while (!s->stop) {
    lk.unlock();
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess) s->hbm_ok.store(free_b >= s->hbm_floor);
    lk.lock();
    s->cond.wait_for(lk, std::chrono::milliseconds(100), [s] { return s->stop; });
  }
}

template <class T>
T* carve(uint8_t*& p, size_t count) {
  T* r = reinterpret_cast<T*>(p);
  p += (count * sizeof(T) + 255) & ~(size_t)255;
  return r;
}

}  // namespace

extern "C" {

int sigops_server_set_variant(sigops_server* s, int variant) {
  if (!s || variant < 0 || variant >= kServeShapes) return SIGOPS_E_INVAL;
  std::lock_guard<std::mutex> g(s->mu);
  s->shape.store(variant, std::memory_order_relaxed);
  s->policy.switch_rate = 0;
  return SIGOPS_OK;
}

int sigops_server_set_adaptive(sigops_server* s, int low_shape, int high_shape, double switch_items_per_s) {
  if (!s || low_shape < 0 || low_shape >= kServeShapes || high_shape < 0 || high_shape >= kServeShapes || !(switch_items_per_s > 0))
    return SIGOPS_E_INVAL;
  std::lock_guard<std::mutex> g(s->mu);
  s->policy.low = low_shape;
  s->policy.high = high_shape;
  s->policy.switch_rate = switch_items_per_s;
  return SIGOPS_OK;
}

int sigops_server_shape_stats(sigops_server* s, int* shape, uint64_t* switches, double* items_per_s) {
  if (!s) return SIGOPS_E_INVAL;
  std::lock_guard<std::mutex> g(s->mu);
  if (shape) *shape = s->running_shape;
  if (switches) *switches = s->shape_switches;
  if (items_per_s) *items_per_s = s->policy.rate;
  return SIGOPS_OK;
}

sigops_server* sigops_server_create(sigops_ctx* ctx, int nslots, size_t slot_items, double hbm_fraction) {
  sg::CtxView v;
  if (!ctx || sg::ctx_view(ctx, &v) != SIGOPS_OK) return nullptr;
  if (nslots <= 0) nslots = 32;
  if (slot_items == 0) slot_items = 16384;
  if (hbm_fraction <= 0 || hbm_fraction > 0.9) hbm_fraction = 0.25;
  if (slot_items > (1u << 20) || (size_t)nslots * slot_items > (1u << 24)) return nullptr;
  cudaSetDevice(v.device);
  size_t free_b = 0, total_b = 0;
  if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) return nullptr;
  std::unique_ptr<sigops_server> s(new sigops_server());
  s->ctx = ctx;
  s->cv = v;
  s->max_items = slot_items;
  s->R = 1u << 16;
  // items in the rings: slots x slot_items, within hbm_fraction of free device
  // memory (a share of the device tile ring per item)
  const size_t per_item_dev = 2 * sizeof(sg::ServeTile) / 32 + 1;
  size_t C = (size_t)nslots * slot_items;
  C = std::min(C, (size_t)(free_b * hbm_fraction) / per_item_dev);
  if (C < slot_items) return nullptr;
  s->C = (uint32_t)C;
  uint32_t cap = 1;
  while (cap < C / 32 + 3ull * std::min<size_t>(s->R, C) + 64) cap <<= 1;  // never the limit before the item ring
  s->tile_cap = cap;
  s->hbm_floor = std::max<size_t>(256ull << 20, total_b / 100);
  // pinned, mapped host rings
  const size_t host_bytes = 4096 + (((size_t)cap * sizeof(sg::ServeTile) + 255) & ~(size_t)255) + ((s->R * 8 + 255) & ~(size_t)255) +
                            C * (64 + 32 + 32 + 64 + 1) + 5 * 256;
  if (sg::host_alloc(&s->host_block, host_bytes, cudaHostAllocMapped | cudaHostAllocPortable) != cudaSuccess) return nullptr;
  memset(s->host_block, 0, host_bytes);
  uint8_t* hp = static_cast<uint8_t*>(s->host_block);
  s->ctl = carve<sg::ServeCtl>(hp, 1);
  hp = static_cast<uint8_t*>(s->host_block) + 4096;
  s->htiles = carve<sg::ServeTile>(hp, cap);
  s->comp = carve<uint64_t>(hp, s->R);
  s->sig = carve<uint8_t>(hp, C * 64);
  s->msg = carve<uint8_t>(hp, C * 32);
  s->pk = carve<uint8_t>(hp, C * 32);
  s->out = carve<uint8_t>(hp, C * 64);
  s->st = carve<uint8_t>(hp, C);
  // device-resident queue
  auto rounded = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t dev_bytes = rounded(sizeof(sg::ServeDev)) + rounded(3 * (size_t)cap * sizeof(sg::ServeTile)) + rounded(s->R * 4);
  if (sg::dev_alloc(&s->dev_block, dev_bytes) != cudaSuccess) {
    sg::host_free(s->host_block);
    s->host_block = nullptr;
    return nullptr;
  }
  uint8_t* dp = static_cast<uint8_t*>(s->dev_block);
  s->dev = carve<sg::ServeDev>(dp, 1);
  s->tiles = carve<sg::ServeTile>(dp, 3 * (size_t)cap);
  s->count = carve<uint32_t>(dp, s->R);
  int block = 0;
  const bool ok = cudaMemset(s->dev_block, 0, dev_bytes) == cudaSuccess &&
                  cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) == cudaSuccess &&
                  cudaStreamCreateWithFlags(&s->stat_stream, cudaStreamNonBlocking) == cudaSuccess &&
                  cudaEventCreateWithFlags(&s->ev_exit, cudaEventDisableTiming) == cudaSuccess && grid_for(s.get(), 0, &block) > 0 &&
                  cudaDeviceSynchronize() == cudaSuccess;
  if (!ok) {
    s->alive = false;
    sigops_server_destroy(s.release());
    return nullptr;
  }
  s->by_slot.resize(s->R);
  s->slot_total.assign(s->R, 0);
  s->handles.reserve(1u << 14);  // in-flight handles of a typical client without a rehash
  sigops_server* p = s.release();
  p->worker = std::thread(worker_loop, p);
  p->monitor = std::thread(monitor_loop, p);
  return p;
}

void sigops_server_destroy(sigops_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> g(s->mu);
    s->stop = true;
  }
  s->cond.notify_all();
  if (s->worker.joinable()) s->worker.join();
  if (s->monitor.joinable()) s->monitor.join();
  cudaSetDevice(s->cv.device);
  if (s->ctl) __atomic_store_n(&s->ctl->stop, 1u, __ATOMIC_RELEASE);  // the kernel closes within microseconds
  if (s->stream) cudaStreamSynchronize(s->stream);
  if (s->ev_exit) cudaEventDestroy(s->ev_exit);
  if (s->stream) cudaStreamDestroy(s->stream);
  if (s->stat_stream) cudaStreamDestroy(s->stat_stream);
  if (s->dev_block) sg::dev_free(s->dev_block);
  if (s->host_block) sg::host_free(s->host_block);
  delete s;
}

size_t sigops_server_slot_items(sigops_server* s) { return s ? s->max_items : 0; }

int sigops_server_submit(sigops_server* s, const uint8_t* curves, int uniform_curve, const uint8_t* sigs, const uint8_t* msgs,
                         const uint8_t* pks, size_t n, uint8_t* out, uint8_t* status, uint64_t* handle) {
  if (!s || !sigs || !msgs || !out || !handle || n == 0) return SIGOPS_E_INVAL;
  if (!curves && (uniform_curve < 0 || uniform_curve > 2)) return SIGOPS_E_INVAL;
  if (!curves && uniform_curve == SIGOPS_ED25519 && !pks) return SIGOPS_E_INVAL;
  if (n > s->max_items) return sg::report(SIGOPS_E_RANGE, "server: request larger than slot_items");
  // items per curve; a request already in curve order is copied as it is
  size_t cnt[3] = {0, 0, 0};
  bool grouped = true;
  if (curves) {
    for (size_t i = 0; i < n; ++i) {
      if (curves[i] > 2) return SIGOPS_E_INVAL;
      cnt[curves[i]]++;
      if (i && curves[i] < curves[i - 1]) grouped = false;
    }
  } else {
    cnt[uniform_curve] = n;
  }
  ReqPtr r = std::make_shared<Request>();
  {
    std::lock_guard<std::mutex> g(s->mu);
    if (!s->alive || s->broken) return sg::report(SIGOPS_E_CUDA, "server: the dispatcher or the kernel has failed");
    if (!s->hbm_ok.load()) return sg::report(SIGOPS_E_BUSY, "server: free device memory below the floor");
    const uint32_t slot = (uint32_t)(s->slots_taken % s->R);
    if (s->by_slot[slot]) return sg::report(SIGOPS_E_BUSY, "server: all request slots in flight");
    // a contiguous run of n items in the rings, wrapping to the start when the end is short
    const uint64_t pos = s->item_tail % s->C;
    const uint64_t skip = pos + n > s->C ? s->C - pos : 0;
    if (s->item_tail - s->item_head + skip + n > s->C) return sg::report(SIGOPS_E_BUSY, "server: item rings full");
    const uint64_t ntiles = (cnt[0] + 31) / 32 + (cnt[1] + 31) / 32 + (cnt[2] + 31) / 32;
    if (s->tile_alloc - s->tile_head + ntiles > s->tile_cap) return sg::report(SIGOPS_E_BUSY, "server: tile rings full");
    r->tile_first = s->tile_alloc;
    s->tile_alloc += ntiles;
    r->tile_end = s->tile_alloc;
    r->id = s->next_id++;
    r->slot = slot;
    r->seq = s->next_seq++;
    r->off = (size_t)((pos + skip) % s->C);
    r->n = n;
    s->item_tail += skip + n;
    r->ring_end = s->item_tail;
    r->out = out;
    r->status = status;
    s->by_slot[slot] = r;
    s->handles[r->id] = r;
    s->slots_taken++;
    s->queued_items += n;
    s->items_in += n;
    *handle = r->id;
  }
  // inputs into the pinned ring grouped by curve (secp256k1, P-256, ed25519),
  // outside the lock: the slot, the items and the tiles are this request's
  const size_t o = r->off;
  if (grouped) {
    memcpy(s->sig + o * 64, sigs, n * 64);
    memcpy(s->msg + o * 32, msgs, n * 32);
    if (pks) memcpy(s->pk + o * 32, pks, n * 32);
    else memset(s->pk + o * 32, 0, n * 32);
  } else {
    r->perm.resize(n);
    size_t pos[3] = {0, cnt[0], cnt[0] + cnt[1]};
    for (size_t i = 0; i < n; ++i) {
      const size_t p = pos[curves[i]]++;
      r->perm[p] = (uint32_t)i;
      memcpy(s->sig + (o + p) * 64, sigs + i * 64, 64);
      memcpy(s->msg + (o + p) * 32, msgs + i * 32, 32);
      if (pks) memcpy(s->pk + (o + p) * 32, pks + i * 32, 32);
      else memset(s->pk + (o + p) * 32, 0, 32);
    }
  }
  // tiles of at most 32 items of one curve; the last one of the request to
  // finish brings the slot's running count to the target
  const uint32_t target = s->slot_total[r->slot] + (uint32_t)n;  // wraps like the device's counter
  s->slot_total[r->slot] = target;
  {
    uint64_t t = r->tile_first;
    size_t base = o;
    for (uint32_t k = 0; k < 3; ++k) {
      for (size_t b = 0; b < cnt[k]; b += 32, ++t) {
        const uint32_t c = (uint32_t)std::min<size_t>(32, cnt[k] - b);
        s->htiles[t % s->tile_cap] = sg::ServeTile{r->slot | (c << 16) | (k << 24), (uint32_t)(base + b), r->seq, target};
      }
      base += cnt[k];
    }
  }
  {
    // publish in submission order: the tile tail advances over the ready prefix
    std::lock_guard<std::mutex> g(s->mu);
    r->ready = true;
    r->t_submit = now_s();
    while (s->published < s->slots_taken) {
      ReqPtr& q = s->by_slot[s->published % s->R];
      if (!q || !q->ready) break;
      if (q->state == RState::Copying) q->state = RState::Running;  // (a request cancelled while copying stays Canceled)
      s->inflight.push_back(q);
      s->published++;
      s->tiles_published = q->tile_end;
    }
    __atomic_store_n(&s->ctl->tile_tail, s->tiles_published, __ATOMIC_RELEASE);
    if (s->broken) fail_inflight(s, SIGOPS_E_CUDA);  // admitted before the kernel failed: nothing will run it
  }
  s->cond.notify_all();
  return SIGOPS_OK;
}

int sigops_server_wait(sigops_server* s, uint64_t handle, int timeout_ms, double* latency_ms) {
  if (!s) return SIGOPS_E_INVAL;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->handles.find(handle);
  if (it == s->handles.end()) return SIGOPS_E_INVAL;
  ReqPtr r = it->second;
  auto pred = [&] { return r->state == RState::Done || r->canceled || !s->alive; };
  // the waiting thread also collects completions (collect_completions)
  std::vector<ReqPtr> finished;
  const auto deadline = Clock::now() + std::chrono::milliseconds(timeout_ms < 0 ? 0 : timeout_ms);
  while (!pred()) {
    collect_completions(s, lk, finished);
    if (s->alive && service_kernel(s, false)) s->cond.notify_all();
    if (pred()) break;
    if (timeout_ms >= 0 && Clock::now() >= deadline) return SIGOPS_E_TIMEDOUT;
    s->cond.wait_for(lk, std::chrono::microseconds(50));
  }
  if (r->canceled) return SIGOPS_E_CANCELED;
  if (r->state != RState::Done) return SIGOPS_E_TIMEDOUT;  // the dispatcher stopped: the request cannot finish
  if (latency_ms) *latency_ms = (r->t_done - r->t_submit) * 1e3;
  s->handles.erase(handle);
  return r->rc;
}

int sigops_server_cancel(sigops_server* s, uint64_t handle) {
  if (!s) return SIGOPS_E_INVAL;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->handles.find(handle);
  if (it == s->handles.end()) return SIGOPS_E_INVAL;
  ReqPtr r = it->second;
  // results being copied into the caller's buffers: let the copy finish
  s->cond.wait(lk, [&] { return r->state != RState::Finishing || !s->alive; });
  if (r->state == RState::Done) return SIGOPS_ALREADY_DONE;
  r->canceled = true;
  if (r->state == RState::Running || r->state == RState::Copying) r->state = RState::Canceled;  // the device still works it off
  s->handles.erase(it);
  s->cond.notify_all();
  return SIGOPS_OK;
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

int sigops_server_kernel_stats(sigops_server* s, uint64_t* tiles, uint64_t* items, double* work_s, double* idle_s, uint64_t* sm_moves) {
  if (!s) return SIGOPS_E_INVAL;
  unsigned long long v[6] = {0, 0, 0, 0, 0, 0};
  cudaSetDevice(s->cv.device);
  if (cudaMemcpyAsync(v, &s->dev->tiles_done, sizeof(v), cudaMemcpyDeviceToHost, s->stat_stream) != cudaSuccess ||
      cudaStreamSynchronize(s->stat_stream) != cudaSuccess)
    return SIGOPS_E_CUDA;
  if (tiles) *tiles = v[0];
  if (items) *items = v[1];
  if (work_s) *work_s = v[2] * 1e-9;
  if (idle_s) *idle_s = v[3] * 1e-9;
  if (sm_moves) *sm_moves = v[4] + v[5];
  return SIGOPS_OK;
}

int sigops_server_dispatch_stats(sigops_server* s, uint64_t* iterations, double* max_gap_ms, double* max_driver_ms) {
  if (!s) return SIGOPS_E_INVAL;
  std::lock_guard<std::mutex> g(s->mu);
  if (iterations) *iterations = s->iterations;
  if (max_gap_ms) *max_gap_ms = s->max_gap * 1e3;
  if (max_driver_ms) *max_driver_ms = s->max_driver * 1e3;
  s->max_gap = 0;
  s->max_driver = 0;
  return SIGOPS_OK;
}

int sigops_server_test_fault(sigops_server* s, int fault) {
  if (!s || fault < 0 || fault > 1) return SIGOPS_E_INVAL;
  {
    std::lock_guard<std::mutex> g(s->mu);
    s->fault = fault;
  }
  s->cond.notify_all();
  return SIGOPS_OK;
}

// Open-loop load: request i covers items [offset[i], offset[i] + count[i]) of
// the pool and is submitted at arrival_s[i] seconds after the start (arrivals
// in non-decreasing order) by client thread i mod kLoadClients, as concurrent
// clients of a server would; the calling thread waits for the requests in
// order, each as soon as it is submitted (and so collects completions while
// the run goes on, as the request threads of a server do).  Outputs land at
// the same item positions.  Fills latency_ms[i] (submit -> results in host
// memory) and the wall time from the start to the last completion.  Returns
// SIGOPS_E_BUSY if admission refused a request (its latency is set to -1).
int sigops_server_run_load(sigops_server* s, const uint8_t* curves, const uint8_t* sigs, const uint8_t* msgs, const uint8_t* pks,
                           const uint64_t* offset, const uint32_t* count, const double* arrival_s, size_t nreq, uint8_t* out,
                           uint8_t* status, double* latency_ms, double* wall_s) {
  if (!s || !curves || !sigs || !msgs || !pks || !offset || !count || !arrival_s || !out || !latency_ms) return SIGOPS_E_INVAL;
  constexpr size_t kLoadClients = 4;
  std::vector<uint64_t> handles(nreq, 0);
  std::unique_ptr<std::atomic<int>[]> state(new std::atomic<int>[nreq]);  // 0 pending, 1 submitted, 2 refused
  for (size_t i = 0; i < nreq; ++i) state[i].store(0);
  {
    // every request of the run is registered before the first wait: size the
    // handle table once, so that no rehash stalls the dispatcher
    std::lock_guard<std::mutex> g(s->mu);
    s->handles.reserve(s->handles.size() + nreq);
  }
  std::atomic<int> rc{SIGOPS_OK};
  auto record = [&](int r) {
    int ok = SIGOPS_OK;
    rc.compare_exchange_strong(ok, r);
  };
  const double t0 = now_s();
  auto client = [&](size_t first) {
    for (size_t i = first; i < nreq; i += kLoadClients) {
      const double target = t0 + arrival_s[i];
      // sleep to the arrival (a client that spins would take a core the dispatcher may need)
      for (double t = now_s(); t < target; t = now_s())
        std::this_thread::sleep_for(std::chrono::microseconds(std::max(1, (int)((target - t) * 1e6))));
      const size_t o = offset[i];
      const int r = sigops_server_submit(s, curves + o, -1, sigs + o * 64, msgs + o * 32, pks + o * 32, count[i], out + o * 64,
                                         status ? status + o : nullptr, &handles[i]);
      if (r != SIGOPS_OK) record(r);
      state[i].store(r == SIGOPS_OK ? 1 : 2, std::memory_order_release);
    }
  };
  std::vector<std::thread> clients;
  for (size_t j = 0; j < std::min(kLoadClients, nreq); ++j) clients.emplace_back(client, j);
  for (size_t i = 0; i < nreq; ++i) {
    int st;
    while ((st = state[i].load(std::memory_order_acquire)) == 0) std::this_thread::sleep_for(std::chrono::microseconds(20));
    if (st == 2) {
      latency_ms[i] = -1;
      continue;
    }
    double lat = 0;
    const int r = sigops_server_wait(s, handles[i], -1, &lat);
    latency_ms[i] = lat;
    if (r != SIGOPS_OK) record(r);
  }
  for (std::thread& c : clients) c.join();
  if (wall_s) *wall_s = now_s() - t0;
  return rc.load();
}

}  // extern "C"
