// Host runtime behind include/sigops.h: contexts, device-resident tables,
// pinned staging, launches and the drop-in entry points.
//
// Replaces the reference's per-call wgpu plumbing (src/gpu.rs:5-186: a new
// instance/adapter/device, pipeline compile and buffers on every call) with a
// resident context: tables are built once, buffers grow and are reused, and a
// call is H2D copy -> one kernel -> D2H copy on the context's stream.
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <atomic>
#include <map>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "../../include/sigops.h"
#include "launch.h"
#include "tables.cuh"

using namespace sg;

namespace {

thread_local std::string g_last_error = "no error";

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

}  // namespace

namespace sg {
int report(int code, const char* what) { return fail(code, "%s", what); }
}  // namespace sg

namespace {

#define SG_CUDA(call)                                                                                 \
  do {                                                                                                \
    cudaError_t e_ = (call);                                                                          \
    if (e_ != cudaSuccess) return fail(SIGOPS_E_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
  } while (0)

// host tables (built once per process)
struct HostTables {
  std::map<std::pair<int, uint32_t>, std::vector<uint32_t>> bases;
  std::mutex mu;
  const std::vector<uint32_t>* get_bases(int curve, uint32_t L) {
    std::lock_guard<std::mutex> g(mu);
    auto key = std::make_pair(curve, L);
    auto it = bases.find(key);
    if (it != bases.end()) return &it->second;
    std::vector<uint32_t> v(bases_len(curve, L));
    if (build_bases(curve, L, v.data()) < 0) return nullptr;
    return &(bases[key] = std::move(v));
  }
};
HostTables& host_tables() {
  static HostTables t;
  return t;
}

bool valid_curve(int c) { return c == SIGOPS_SECP256K1 || c == SIGOPS_SECP256R1 || c == SIGOPS_ED25519; }
bool valid_L(uint32_t L) { return L >= MIN_LOG_LIMB && L <= MAX_LOG_LIMB; }

}  // namespace

namespace sg {

// allocations that the failure-injection hook may refuse
static std::atomic<int> g_fail_allocs{0};

static bool take_injected_failure() {
  int v = g_fail_allocs.load();
  while (v > 0)
    if (g_fail_allocs.compare_exchange_weak(v, v - 1)) return true;
  return false;
}

cudaError_t dev_alloc(void** p, size_t bytes) {
  *p = nullptr;
  if (take_injected_failure()) return cudaErrorMemoryAllocation;
  return cudaMalloc(p, bytes);
}
void dev_free(void* p) {
  if (p) cudaFree(p);
}
cudaError_t host_alloc(void** p, size_t bytes, unsigned flags) {
  *p = nullptr;
  if (take_injected_failure()) return cudaErrorMemoryAllocation;
  return cudaHostAlloc(p, bytes, flags);
}
void host_free(void* p) {
  if (p) cudaFreeHost(p);
}

}  // namespace sg

struct sigops_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  int num_sms = 0;
  int grid[3] = {0, 0, 0};     // plain kernels: blocks per launch, per curve
  int variant[3] = {0, 0, 0};  // plain kernel variant per curve
  uint32_t* d_gtab[3] = {nullptr, nullptr, nullptr};
  uint32_t* d_gsmall[3] = {nullptr, nullptr, nullptr};  // 8-bit-window tables (staged into shared memory by the kernels)
  uint32_t* d_err = nullptr;
  uint8_t* d_buf = nullptr;  // inputs then outputs of host-buffer calls
  size_t d_cap = 0;
  uint8_t* h_buf = nullptr;  // pinned staging
  size_t h_cap = 0;
  // batched engine
  void* d_scratch = nullptr;  // Scratch record
  uint32_t* d_idx = nullptr;  // 3 * idx_cap per-curve index lists
  uint8_t* d_defer = nullptr;  // batched_defer_bytes(idx_cap): shared-inversion scratch of the single-curve variants
  size_t idx_cap = 0;
  int batched_variant = 0;
  int batched_grid = 0;
  ForkStreams fork{};  // side streams of the single-curve batched variants
  // first half of a pipelined sigops_verify_mixed: its own stream and side
  // streams at the highest priority, its own scratch record (the index lists
  // split the one allocation)
  cudaStream_t stream2 = nullptr;
  ForkStreams fork2{};
  void* d_scratch2 = nullptr;
  cudaEvent_t ev_order = nullptr, ev_join = nullptr;
  std::mutex mu;
};

struct sigops_plan {
  sigops_ctx* ctx = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

namespace {

int ensure_buffers(sigops_ctx* c, size_t bytes) {
  bytes = (bytes + 255) & ~(size_t)255;
  if (bytes > c->d_cap) {
    dev_free(c->d_buf);
    c->d_buf = nullptr;
    c->d_cap = 0;
    if (dev_alloc((void**)&c->d_buf, bytes) != cudaSuccess) return fail(SIGOPS_E_NOMEM, "cudaMalloc(%zu) failed", bytes);
    c->d_cap = bytes;
  }
  if (bytes > c->h_cap) {
    host_free(c->h_buf);
    c->h_buf = nullptr;
    c->h_cap = 0;
    if (host_alloc((void**)&c->h_buf, bytes) != cudaSuccess) return fail(SIGOPS_E_NOMEM, "cudaMallocHost(%zu) failed", bytes);
    c->h_cap = bytes;
  }
  return SIGOPS_OK;
}

int ensure_device(sigops_ctx* c, size_t bytes) {
  bytes = (bytes + 255) & ~(size_t)255;
  if (bytes <= c->d_cap) return SIGOPS_OK;
  dev_free(c->d_buf);
  c->d_buf = nullptr;
  c->d_cap = 0;
  if (dev_alloc((void**)&c->d_buf, bytes) != cudaSuccess) return fail(SIGOPS_E_NOMEM, "cudaMalloc(%zu) failed", bytes);
  c->d_cap = bytes;
  return SIGOPS_OK;
}

bool is_pinned(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

int ensure_idx(sigops_ctx* c, size_t n) {
  if (n <= c->idx_cap) return SIGOPS_OK;
  dev_free(c->d_idx);
  dev_free(c->d_defer);
  c->d_idx = nullptr;
  c->d_defer = nullptr;
  c->idx_cap = 0;
  if (dev_alloc((void**)&c->d_idx, 3 * n * sizeof(uint32_t)) != cudaSuccess) return fail(SIGOPS_E_NOMEM, "cudaMalloc(index lists, %zu)", n);
  if (dev_alloc((void**)&c->d_defer, batched_defer_bytes(n)) != cudaSuccess) {
    dev_free(c->d_idx);
    c->d_idx = nullptr;
    return fail(SIGOPS_E_NOMEM, "cudaMalloc(inversion scratch, %zu)", n);
  }
  c->idx_cap = n;
  return SIGOPS_OK;
}

// kernel 0..2: plain kernel of that curve; 3: batched engine
int set_variant(sigops_ctx* c, int kernel, int variant) {
  if (kernel >= 0 && kernel < 3) {
    if (variant < 0 || variant >= PLAIN_VARIANTS) return fail(SIGOPS_E_INVAL, "plain variant %d out of range", variant);
    int bps = plain_max_blocks_per_sm(kernel, variant);
    if (bps <= 0) return fail(SIGOPS_E_CUDA, "plain kernel %d variant %d cannot launch", kernel, variant);
    c->variant[kernel] = variant;
    c->grid[kernel] = c->num_sms * bps;
    return SIGOPS_OK;
  }
  if (kernel == 3) {
    if (variant < 0 || variant >= BATCHED_VARIANTS) return fail(SIGOPS_E_INVAL, "batched variant %d out of range", variant);
    int bps = batched_max_blocks_per_sm(variant);
    if (bps <= 0) return fail(SIGOPS_E_CUDA, "batched variant %d cannot launch", variant);
    c->batched_variant = variant;
    c->batched_grid = c->num_sms * bps;
    return SIGOPS_OK;
  }
  return fail(SIGOPS_E_INVAL, "kernel id %d out of range", kernel);
}

cudaError_t launch_mixed_on(sigops_ctx* c, const uint8_t* curves, const uint8_t* sigs, const uint8_t* msgs, const uint8_t* pks, size_t n,
                            uint8_t* out, uint8_t* status, uint32_t* idx, void* scratch, void* defer, const ForkStreams* fork,
                            cudaStream_t s) {
  size_t cg = (n + 255) / 256;
  int classify_grid = (int)(cg < (size_t)c->num_sms * 8 ? cg : (size_t)c->num_sms * 8);
  const GenTables tabs{{c->d_gtab[0], c->d_gtab[1], c->d_gtab[2]}, {c->d_gsmall[0], c->d_gsmall[1], c->d_gsmall[2]}};
  return launch_batched(curves, sigs, msgs, pks, n, out, status, idx, scratch, defer, tabs, c->d_err, c->batched_grid, c->batched_variant,
                        classify_grid, fork, s);
}

cudaError_t launch_mixed(sigops_ctx* c, const uint8_t* curves, const uint8_t* sigs, const uint8_t* msgs, const uint8_t* pks, size_t n,
                         uint8_t* out, uint8_t* status, cudaStream_t s) {
  return launch_mixed_on(c, curves, sigs, msgs, pks, n, out, status, c->d_idx, c->d_scratch, c->d_defer, &c->fork, s);
}

int check_device_errors(sigops_ctx* c) {
  uint32_t e = 0;
  SG_CUDA(cudaMemcpyAsync(&e, c->d_err, sizeof e, cudaMemcpyDeviceToHost, c->stream));
  SG_CUDA(cudaStreamSynchronize(c->stream));
  if (e) {
    SG_CUDA(cudaMemsetAsync(c->d_err, 0, sizeof(uint32_t), c->stream));
    SG_CUDA(cudaStreamSynchronize(c->stream));
    if (e & DEV_ERR_WAIT_TIMEOUT) return fail(SIGOPS_E_TIMEDOUT, "device: bounded wait expired (error bits 0x%x)", e);
    return fail(SIGOPS_E_TIMEDOUT, "device error bits 0x%x", e);
  }
  return SIGOPS_OK;
}

std::mutex g_default_mu;
sigops_ctx* g_default = nullptr;

sigops_ctx* resolve(sigops_ctx* c) {
  if (c) return c;
  std::lock_guard<std::mutex> g(g_default_mu);
  if (!g_default) g_default = sigops_create(0);
  return g_default;
}

// layout of the staging buffer for one host-buffer call
struct Layout {
  size_t sig, msg, pk, out, status, total;
};
Layout layout_for(int curve, size_t n) {
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  Layout l;
  l.sig = 0;
  l.msg = al(l.sig + n * 64);
  l.pk = al(l.msg + n * 32);
  size_t after_pk = curve == SIGOPS_ED25519 ? al(l.pk + n * 32) : l.pk;
  l.out = after_pk;
  l.status = al(l.out + (curve == SIGOPS_ED25519 ? n : n * 64));
  l.total = al(l.status + n);
  return l;
}

// The plain kernel of `curve` for a batch of n: the tuned launch variant, or
// for a batch too small to fill the GPU, one-warp blocks spread over the SMs
// (secp256k1 with a lane pair per signature while few warps are needed)
cudaError_t launch_plain_for(sigops_ctx* c, int curve, const uint8_t* sigs, const uint8_t* msgs, const uint8_t* pks, size_t n, uint8_t* out,
                             uint8_t* status, cudaStream_t stream) {
  if (plain_small_batch(n, c->num_sms))
    return launch_plain_small(curve, sigs, msgs, pks, n, c->d_gtab[curve], out, status, c->d_err, c->num_sms, stream);
  return launch_plain(curve, sigs, msgs, pks, n, c->d_gtab[curve], out, status, c->d_err, c->variant[curve], stream);
}

int run_host_call(sigops_ctx* ctx, int curve, const uint8_t* sigs, const uint8_t* msgs, const uint8_t* pks, size_t n, uint8_t* out,
                  uint8_t* out_status) {
  if (n == 0) return SIGOPS_OK;
  if (!sigs || !msgs || !out || (curve == SIGOPS_ED25519 && !pks)) return fail(SIGOPS_E_INVAL, "null buffer");
  sigops_ctx* c = resolve(ctx);
  if (!c) return SIGOPS_E_NODEV;
  std::lock_guard<std::mutex> g(c->mu);
  SG_CUDA(cudaSetDevice(c->device));
  Layout l = layout_for(curve, n);
  int rc = ensure_buffers(c, l.total);
  if (rc) return rc;
  memcpy(c->h_buf + l.sig, sigs, n * 64);
  memcpy(c->h_buf + l.msg, msgs, n * 32);
  if (curve == SIGOPS_ED25519) memcpy(c->h_buf + l.pk, pks, n * 32);
  SG_CUDA(cudaMemcpyAsync(c->d_buf, c->h_buf, l.out, cudaMemcpyHostToDevice, c->stream));
  SG_CUDA(launch_plain_for(c, curve, c->d_buf + l.sig, c->d_buf + l.msg, c->d_buf + l.pk, n, c->d_buf + l.out, c->d_buf + l.status,
                           c->stream));
  SG_CUDA(cudaMemcpyAsync(c->h_buf + l.out, c->d_buf + l.out, l.total - l.out, cudaMemcpyDeviceToHost, c->stream));
  rc = check_device_errors(c);
  if (rc) return rc;
  memcpy(out, c->h_buf + l.out, curve == SIGOPS_ED25519 ? n : n * 64);
  if (out_status) memcpy(out_status, c->h_buf + l.status, n);
  return SIGOPS_OK;
}

int check_table_arg(int curve, const uint32_t* table, size_t len, uint32_t L) {
  if (!table && len) return fail(SIGOPS_E_INVAL, "null table_limbs");
  return sigops_check_table(curve, table, len, L);
}

}  // namespace

namespace sg {
int ctx_view(sigops_ctx* c, CtxView* v) {
  if (!c || !v) return SIGOPS_E_INVAL;
  v->device = c->device;
  v->num_sms = c->num_sms;
  for (int k = 0; k < 3; ++k) {
    v->gtab[k] = c->d_gtab[k];
    v->tabs.big[k] = c->d_gtab[k];
    v->tabs.small[k] = c->d_gsmall[k];
  }
  v->d_err = c->d_err;
  v->batched_grid = c->batched_grid;
  v->batched_variant = c->batched_variant;
  return SIGOPS_OK;
}
}  // namespace sg

extern "C" {

const char* sigops_version(void) { return "sigops-gb300 0.1 (sm_103a)"; }

const char* sigops_last_error(void) { return g_last_error.c_str(); }

const char* sigops_strerror(int code) {
  switch (code) {
    case SIGOPS_OK: return "ok";
    case SIGOPS_E_INVAL: return "invalid argument";
    case SIGOPS_E_NOMEM: return "out of memory";
    case SIGOPS_E_NODEV: return "no such CUDA device";
    case SIGOPS_E_CUDA: return "CUDA error";
    case SIGOPS_E_TABLE: return "table_limbs do not match the generator table";
    case SIGOPS_E_TIMEDOUT: return "device wait timed out";
    case SIGOPS_E_BUSY: return "busy";
    case SIGOPS_E_RANGE: return "batch exceeds capacity";
    case SIGOPS_E_CANCELED: return "request cancelled";
    case SIGOPS_ALREADY_DONE: return "request already finished";
    default: return "unknown error";
  }
}

sigops_ctx* sigops_create(int device) {
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
    fail(SIGOPS_E_NODEV, "no CUDA device %d (count %d)", device, ndev);
    return nullptr;
  }
  const KernelTables& tabs = kernel_tables();
  sigops_ctx* c = new sigops_ctx();
  c->device = device;
  auto bail = [&](const char* what, cudaError_t e) -> sigops_ctx* {
    fail(SIGOPS_E_CUDA, "%s: %s", what, cudaGetErrorString(e));
    sigops_destroy(c);
    return nullptr;
  };
  cudaError_t e;
  if ((e = cudaSetDevice(device)) != cudaSuccess) return bail("cudaSetDevice", e);
  if ((e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) != cudaSuccess) return bail("cudaStreamCreate", e);
  if ((e = fork_streams_create(&c->fork)) != cudaSuccess) return bail("side streams", e);
  int prio_least = 0, prio_greatest = 0;
  if ((e = cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest)) != cudaSuccess) return bail("stream priorities", e);
  if ((e = cudaStreamCreateWithPriority(&c->stream2, cudaStreamNonBlocking, prio_greatest)) != cudaSuccess) return bail("cudaStreamCreate", e);
  if ((e = fork_streams_create(&c->fork2, prio_greatest)) != cudaSuccess) return bail("side streams", e);
  if ((e = cudaEventCreateWithFlags(&c->ev_order, cudaEventDisableTiming)) != cudaSuccess) return bail("cudaEventCreate", e);
  if ((e = cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming)) != cudaSuccess) return bail("cudaEventCreate", e);
  if ((e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device)) != cudaSuccess) return bail("attr", e);
  for (int k = 0; k < 3; ++k) {
    const auto& t = tabs.tab[k];
    if ((e = dev_alloc((void**)&c->d_gtab[k], t.size() * 4)) != cudaSuccess) return bail("cudaMalloc(table)", e);
    if ((e = cudaMemcpy(c->d_gtab[k], t.data(), t.size() * 4, cudaMemcpyHostToDevice)) != cudaSuccess) return bail("table upload", e);
    const auto& sm = tabs.small[k];
    if ((e = dev_alloc((void**)&c->d_gsmall[k], sm.size() * 4)) != cudaSuccess) return bail("cudaMalloc(table)", e);
    if ((e = cudaMemcpy(c->d_gsmall[k], sm.data(), sm.size() * 4, cudaMemcpyHostToDevice)) != cudaSuccess) return bail("table upload", e);
    if (set_variant(c, k, 0) != SIGOPS_OK) {
      sigops_destroy(c);
      return nullptr;
    }
  }
  if ((e = dev_alloc((void**)&c->d_err, sizeof(uint32_t))) != cudaSuccess) return bail("cudaMalloc(err)", e);
  if ((e = dev_alloc(&c->d_scratch, batched_scratch_bytes())) != cudaSuccess) return bail("cudaMalloc(scratch)", e);
  if ((e = dev_alloc(&c->d_scratch2, batched_scratch_bytes())) != cudaSuccess) return bail("cudaMalloc(scratch)", e);
  if (set_variant(c, 3, 0) != SIGOPS_OK) {
    sigops_destroy(c);
    return nullptr;
  }
  int tuned[4];
  if (tune_cache_lookup(device, tuned))  // a previous sigops_autotune on this device model
    for (int k = 0; k < 4; ++k) set_variant(c, k, tuned[k]);
  if ((e = cudaMemset(c->d_err, 0, sizeof(uint32_t))) != cudaSuccess) return bail("memset", e);
  return c;
}

void sigops_destroy(sigops_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->stream2) cudaStreamSynchronize(c->stream2);
  for (int k = 0; k < 3; ++k) {
    dev_free(c->d_gtab[k]);
    dev_free(c->d_gsmall[k]);
  }
  dev_free(c->d_err);
  dev_free(c->d_scratch);
  dev_free(c->d_scratch2);
  dev_free(c->d_idx);
  dev_free(c->d_defer);
  dev_free(c->d_buf);
  host_free(c->h_buf);
  if (c->stream) cudaStreamDestroy(c->stream);
  fork_streams_destroy(&c->fork);
  if (c->stream2) cudaStreamDestroy(c->stream2);
  fork_streams_destroy(&c->fork2);
  if (c->ev_order) cudaEventDestroy(c->ev_order);
  if (c->ev_join) cudaEventDestroy(c->ev_join);
  {
    std::lock_guard<std::mutex> g(g_default_mu);
    if (g_default == c) g_default = nullptr;
  }
  delete c;
}

long sigops_bases_len(int curve, uint32_t L) {
  if (!valid_curve(curve) || !valid_L(L)) return fail(SIGOPS_E_INVAL, "bad curve %d or log_limb_size %u", curve, L);
  return bases_len(curve, L);
}

long sigops_bases(int curve, uint32_t L, uint32_t* out, size_t cap) {
  long len = sigops_bases_len(curve, L);
  if (len < 0) return len;
  if (!out || cap < (size_t)len) return fail(SIGOPS_E_INVAL, "output capacity %zu < %ld", cap, len);
  const std::vector<uint32_t>* v = host_tables().get_bases(curve, L);
  if (!v) return fail(SIGOPS_E_INVAL, "table build failed");
  memcpy(out, v->data(), v->size() * 4);
  return len;
}

int sigops_check_table(int curve, const uint32_t* table, size_t len, uint32_t L) {
  long want = sigops_bases_len(curve, L);
  if (want < 0) return (int)want;
  const std::vector<uint32_t>* v = host_tables().get_bases(curve, L);
  if (!v) return fail(SIGOPS_E_INVAL, "table build failed");
  if (len != (size_t)want || !table || memcmp(table, v->data(), len * 4) != 0)
    return fail(SIGOPS_E_TABLE, "table_limbs differ from precompute bases (len %zu, expected %ld)", len, want);
  return SIGOPS_OK;
}

int sigops_secp256k1_ecrecover(sigops_ctx* ctx, const uint8_t* sigs, const uint8_t* msgs, size_t n, const uint32_t* table,
                               size_t table_len, uint32_t L, uint8_t* out, uint8_t* status) {
  int rc = check_table_arg(SIGOPS_SECP256K1, table, table_len, L);
  if (rc) return rc;
  return run_host_call(ctx, SIGOPS_SECP256K1, sigs, msgs, nullptr, n, out, status);
}

int sigops_secp256k1_ecrecover_single_shader(sigops_ctx* ctx, const uint8_t* sigs, const uint8_t* msgs, size_t n, uint32_t L,
                                             uint8_t* out, uint8_t* status) {
  if (!valid_L(L)) return fail(SIGOPS_E_INVAL, "log_limb_size %u outside [11, 15]", L);
  return run_host_call(ctx, SIGOPS_SECP256K1, sigs, msgs, nullptr, n, out, status);
}

int sigops_secp256r1_ecrecover(sigops_ctx* ctx, const uint8_t* sigs, const uint8_t* msgs, size_t n, const uint32_t* table,
                               size_t table_len, uint32_t L, uint8_t* out, uint8_t* status) {
  int rc = check_table_arg(SIGOPS_SECP256R1, table, table_len, L);
  if (rc) return rc;
  return run_host_call(ctx, SIGOPS_SECP256R1, sigs, msgs, nullptr, n, out, status);
}

int sigops_secp256r1_ecrecover_single_shader(sigops_ctx* ctx, const uint8_t* sigs, const uint8_t* msgs, size_t n, uint32_t L,
                                             uint8_t* out, uint8_t* status) {
  if (!valid_L(L)) return fail(SIGOPS_E_INVAL, "log_limb_size %u outside [11, 15]", L);
  return run_host_call(ctx, SIGOPS_SECP256R1, sigs, msgs, nullptr, n, out, status);
}

int sigops_ed25519_ecverify(sigops_ctx* ctx, const uint8_t* sigs, const uint8_t* msgs, const uint8_t* pks, size_t n,
                            const uint32_t* table, size_t table_len, uint32_t L, uint8_t* valid, uint8_t* status) {
  int rc = check_table_arg(SIGOPS_ED25519, table, table_len, L);
  if (rc) return rc;
  return run_host_call(ctx, SIGOPS_ED25519, sigs, msgs, pks, n, valid, status);
}

int sigops_ed25519_ecverify_single(sigops_ctx* ctx, const uint8_t* sigs, const uint8_t* msgs, const uint8_t* pks, size_t n, uint32_t L,
                                   uint8_t* valid, uint8_t* status) {
  if (!valid_L(L)) return fail(SIGOPS_E_INVAL, "log_limb_size %u outside [11, 15]", L);
  return run_host_call(ctx, SIGOPS_ED25519, sigs, msgs, pks, n, valid, status);
}

int sigops_ed25519_verify_raw(sigops_ctx* ctx, const uint8_t* sigs, const uint8_t* msgs, size_t msgs_bytes, const uint64_t* msg_offsets,
                              const uint32_t* msg_lens, const uint8_t* pks, size_t n, uint8_t* valid, uint8_t* status) {
  if (n == 0) return SIGOPS_OK;
  if (!sigs || !msg_offsets || !msg_lens || !pks || !valid || (!msgs && msgs_bytes)) return fail(SIGOPS_E_INVAL, "null buffer");
  for (size_t i = 0; i < n; ++i)
    if (msg_offsets[i] > msgs_bytes || msg_lens[i] > msgs_bytes - msg_offsets[i])
      return fail(SIGOPS_E_INVAL, "message %zu (offset %llu, %u bytes) runs past the %zu message bytes", i,
                  (unsigned long long)msg_offsets[i], msg_lens[i], msgs_bytes);
  sigops_ctx* c = resolve(ctx);
  if (!c) return SIGOPS_E_NODEV;
  std::lock_guard<std::mutex> g(c->mu);
  SG_CUDA(cudaSetDevice(c->device));
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  const size_t o_sig = 0, o_pk = al(n * 64), o_off = o_pk + al(n * 32), o_len = o_off + al(n * 8), o_msg = o_len + al(n * 4),
               o_out = o_msg + al(msgs_bytes ? msgs_bytes : 1), o_st = o_out + al(n), total = o_st + al(n);
  int rc = ensure_buffers(c, total);
  if (rc) return rc;
  memcpy(c->h_buf + o_sig, sigs, n * 64);
  memcpy(c->h_buf + o_pk, pks, n * 32);
  memcpy(c->h_buf + o_off, msg_offsets, n * 8);
  memcpy(c->h_buf + o_len, msg_lens, n * 4);
  if (msgs_bytes) memcpy(c->h_buf + o_msg, msgs, msgs_bytes);
  SG_CUDA(cudaMemcpyAsync(c->d_buf, c->h_buf, o_out, cudaMemcpyHostToDevice, c->stream));
  SG_CUDA(launch_raw_ed(c->d_buf + o_sig, c->d_buf + o_msg, (const uint64_t*)(c->d_buf + o_off), (const uint32_t*)(c->d_buf + o_len),
                        c->d_buf + o_pk, n, c->d_gtab[SIGOPS_ED25519], c->d_buf + o_out, c->d_buf + o_st, c->d_err,
                        c->variant[SIGOPS_ED25519], c->stream));
  SG_CUDA(cudaMemcpyAsync(c->h_buf + o_out, c->d_buf + o_out, total - o_out, cudaMemcpyDeviceToHost, c->stream));
  rc = check_device_errors(c);
  if (rc) return rc;
  memcpy(valid, c->h_buf + o_out, n);
  if (status) memcpy(status, c->h_buf + o_st, n);
  return SIGOPS_OK;
}

int sigops_plain_device(sigops_ctx* ctx, int curve, const uint8_t* d_sigs, const uint8_t* d_msgs, const uint8_t* d_pks, size_t n,
                        uint8_t* d_out, uint8_t* d_status, void* stream) {
  if (!valid_curve(curve)) return fail(SIGOPS_E_INVAL, "bad curve %d", curve);
  if (n == 0) return SIGOPS_OK;
  auto misaligned = [](const void* p) { return ((uintptr_t)p & 15u) != 0; };
  if (!d_sigs || !d_msgs || !d_out || !d_status || (curve == SIGOPS_ED25519 && !d_pks))
    return fail(SIGOPS_E_INVAL, "null device buffer");
  if (misaligned(d_sigs) || misaligned(d_msgs) || misaligned(d_out) || (curve == SIGOPS_ED25519 && misaligned(d_pks)))
    return fail(SIGOPS_E_INVAL, "device buffers must be 16-byte aligned");
  sigops_ctx* c = resolve(ctx);
  if (!c) return SIGOPS_E_NODEV;
  std::lock_guard<std::mutex> g(c->mu);
  SG_CUDA(cudaSetDevice(c->device));
  cudaStream_t s = stream ? (cudaStream_t)stream : c->stream;
  SG_CUDA(launch_plain_for(c, curve, d_sigs, d_msgs, d_pks, n, d_out, d_status, s));
  return SIGOPS_OK;
}

int sigops_reserve(sigops_ctx* ctx, size_t n) {
  sigops_ctx* c = resolve(ctx);
  if (!c) return SIGOPS_E_NODEV;
  std::lock_guard<std::mutex> g(c->mu);
  SG_CUDA(cudaSetDevice(c->device));
  return ensure_idx(c, n);
}

// largest batch of the mixed engine (32-bit item indices)
constexpr size_t kMaxMixedItems = 0xffffffffull;

int sigops_verify_mixed_device(sigops_ctx* ctx, const uint8_t* d_curves, const uint8_t* d_sigs, const uint8_t* d_msgs, const uint8_t* d_pks,
                               size_t n, uint8_t* d_out, uint8_t* d_status, void* stream) {
  if (n > kMaxMixedItems) return fail(SIGOPS_E_RANGE, "batch of %zu items: the index lists hold 32-bit indices", n);
  if (n == 0) return SIGOPS_OK;
  auto misaligned = [](const void* p) { return ((uintptr_t)p & 15u) != 0; };
  if (!d_curves || !d_sigs || !d_msgs || !d_pks || !d_out || !d_status) return fail(SIGOPS_E_INVAL, "null device buffer");
  if (misaligned(d_sigs) || misaligned(d_msgs) || misaligned(d_pks) || misaligned(d_out))
    return fail(SIGOPS_E_INVAL, "device buffers must be 16-byte aligned");
  sigops_ctx* c = resolve(ctx);
  if (!c) return SIGOPS_E_NODEV;
  std::lock_guard<std::mutex> g(c->mu);
  SG_CUDA(cudaSetDevice(c->device));
  int rc = ensure_idx(c, n);
  if (rc) return rc;
  SG_CUDA(launch_mixed(c, d_curves, d_sigs, d_msgs, d_pks, n, d_out, d_status, stream ? (cudaStream_t)stream : c->stream));
  return SIGOPS_OK;
}

// page-locked calls from this size on run as two pipelined halves
constexpr size_t kPipelineMin = 131072;

int sigops_verify_mixed(sigops_ctx* ctx, const uint8_t* curves, const uint8_t* sigs, const uint8_t* msgs, const uint8_t* pks, size_t n,
                        uint8_t* out, uint8_t* out_status) {
  if (n > kMaxMixedItems) return fail(SIGOPS_E_RANGE, "batch of %zu items: the index lists hold 32-bit indices", n);
  if (n == 0) return SIGOPS_OK;
  if (!curves || !sigs || !msgs || !pks || !out) return fail(SIGOPS_E_INVAL, "null buffer");
  {
    // the largest tag (a loop the compiler vectorises) decides; the index of
    // the first bad tag is only searched for the error message
    uint8_t top = 0;
    for (size_t i = 0; i < n; ++i) top = curves[i] > top ? curves[i] : top;
    if (top > 2)
      for (size_t i = 0; i < n; ++i)
        if (curves[i] > 2) return fail(SIGOPS_E_INVAL, "item %zu has unknown curve tag %u", i, (unsigned)curves[i]);
  }
  sigops_ctx* c = resolve(ctx);
  if (!c) return SIGOPS_E_NODEV;
  std::lock_guard<std::mutex> g(c->mu);
  SG_CUDA(cudaSetDevice(c->device));
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  const size_t o_sig = 0, o_msg = al(n * 64), o_pk = o_msg + al(n * 32), o_cur = o_pk + al(n * 32), o_out = o_cur + al(n),
               o_st = o_out + al(n * 64), total = o_st + al(n);
  // caller buffers that are page-locked go straight to / from the device
  const bool pinned = is_pinned(sigs) && is_pinned(msgs) && is_pinned(pks) && is_pinned(curves) && is_pinned(out) &&
                      (!out_status || is_pinned(out_status));
  int rc = pinned ? ensure_device(c, total) : ensure_buffers(c, total);
  if (rc) return rc;
  rc = ensure_idx(c, n);
  if (rc) return rc;
  if (pinned && n >= kPipelineMin) {
    // two halves on two streams: the first on the high-priority stream, so
    // its blocks go first and the second half's fill the SMs it leaves idle;
    // the second half's inputs cross while the first half computes, and the
    // first half's results cross while the second half computes
    const size_t half = (n / 2 + 255) & ~(size_t)255;
    SG_CUDA(cudaEventRecord(c->ev_order, c->stream));  // after any earlier work on the buffers
    SG_CUDA(cudaStreamWaitEvent(c->stream2, c->ev_order, 0));
    for (int k = 0; k < 2; ++k) {
      const size_t b = k ? half : 0, m = k ? n - half : half;
      cudaStream_t s = k ? c->stream : c->stream2;
      SG_CUDA(cudaMemcpyAsync(c->d_buf + o_sig + b * 64, sigs + b * 64, m * 64, cudaMemcpyHostToDevice, s));
      SG_CUDA(cudaMemcpyAsync(c->d_buf + o_msg + b * 32, msgs + b * 32, m * 32, cudaMemcpyHostToDevice, s));
      SG_CUDA(cudaMemcpyAsync(c->d_buf + o_pk + b * 32, pks + b * 32, m * 32, cudaMemcpyHostToDevice, s));
      SG_CUDA(cudaMemcpyAsync(c->d_buf + o_cur + b, curves + b, m, cudaMemcpyHostToDevice, s));
      SG_CUDA(launch_mixed_on(c, c->d_buf + o_cur + b, c->d_buf + o_sig + b * 64, c->d_buf + o_msg + b * 32, c->d_buf + o_pk + b * 32, m,
                              c->d_buf + o_out + b * 64, c->d_buf + o_st + b, c->d_idx + (k ? 3 * half : 0),
                              k ? c->d_scratch : c->d_scratch2, c->d_defer + (k ? batched_defer_bytes(half) : 0),
                              k ? &c->fork : &c->fork2, s));
      SG_CUDA(cudaMemcpyAsync(out + b * 64, c->d_buf + o_out + b * 64, m * 64, cudaMemcpyDeviceToHost, s));
      if (out_status) SG_CUDA(cudaMemcpyAsync(out_status + b, c->d_buf + o_st + b, m, cudaMemcpyDeviceToHost, s));
    }
    SG_CUDA(cudaEventRecord(c->ev_join, c->stream2));
    SG_CUDA(cudaStreamWaitEvent(c->stream, c->ev_join, 0));
    return check_device_errors(c);
  }
  if (pinned) {
    SG_CUDA(cudaMemcpyAsync(c->d_buf + o_sig, sigs, n * 64, cudaMemcpyHostToDevice, c->stream));
    SG_CUDA(cudaMemcpyAsync(c->d_buf + o_msg, msgs, n * 32, cudaMemcpyHostToDevice, c->stream));
    SG_CUDA(cudaMemcpyAsync(c->d_buf + o_pk, pks, n * 32, cudaMemcpyHostToDevice, c->stream));
    SG_CUDA(cudaMemcpyAsync(c->d_buf + o_cur, curves, n, cudaMemcpyHostToDevice, c->stream));
  } else {
    memcpy(c->h_buf + o_sig, sigs, n * 64);
    memcpy(c->h_buf + o_msg, msgs, n * 32);
    memcpy(c->h_buf + o_pk, pks, n * 32);
    memcpy(c->h_buf + o_cur, curves, n);
    SG_CUDA(cudaMemcpyAsync(c->d_buf, c->h_buf, o_out, cudaMemcpyHostToDevice, c->stream));
  }
  SG_CUDA(launch_mixed(c, c->d_buf + o_cur, c->d_buf + o_sig, c->d_buf + o_msg, c->d_buf + o_pk, n, c->d_buf + o_out, c->d_buf + o_st,
                       c->stream));
  if (pinned) {
    SG_CUDA(cudaMemcpyAsync(out, c->d_buf + o_out, n * 64, cudaMemcpyDeviceToHost, c->stream));
    if (out_status) SG_CUDA(cudaMemcpyAsync(out_status, c->d_buf + o_st, n, cudaMemcpyDeviceToHost, c->stream));
    return check_device_errors(c);
  }
  SG_CUDA(cudaMemcpyAsync(c->h_buf + o_out, c->d_buf + o_out, total - o_out, cudaMemcpyDeviceToHost, c->stream));
  rc = check_device_errors(c);
  if (rc) return rc;
  memcpy(out, c->h_buf + o_out, n * 64);
  if (out_status) memcpy(out_status, c->h_buf + o_st, n);
  return SIGOPS_OK;
}

int sigops_mixed_plan_create(sigops_ctx* ctx, const uint8_t* d_curves, const uint8_t* d_sigs, const uint8_t* d_msgs, const uint8_t* d_pks,
                             size_t n, uint8_t* d_out, uint8_t* d_status, sigops_plan** plan_out) {
  if (n > kMaxMixedItems) return fail(SIGOPS_E_RANGE, "batch of %zu items: the index lists hold 32-bit indices", n);
  if (!plan_out || n == 0) return fail(SIGOPS_E_INVAL, "plan needs n > 0 and an output pointer");
  sigops_ctx* c = resolve(ctx);
  if (!c) return SIGOPS_E_NODEV;
  std::lock_guard<std::mutex> g(c->mu);
  SG_CUDA(cudaSetDevice(c->device));
  int rc = ensure_idx(c, n);
  if (rc) return rc;
  sigops_plan* p = new sigops_plan();
  p->ctx = c;
  cudaStream_t cs;
  SG_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    cudaError_t le = launch_mixed(c, d_curves, d_sigs, d_msgs, d_pks, n, d_out, d_status, cs);
    e = cudaStreamEndCapture(cs, &p->graph);
    if (le != cudaSuccess) e = le;
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&p->exec, p->graph, 0);
  cudaStreamDestroy(cs);
  if (e != cudaSuccess) {
    if (p->graph) cudaGraphDestroy(p->graph);
    delete p;
    return fail(SIGOPS_E_CUDA, "graph capture failed: %s", cudaGetErrorString(e));
  }
  *plan_out = p;
  return SIGOPS_OK;
}

int sigops_mixed_plan_launch(sigops_plan* p, void* stream) {
  if (!p) return fail(SIGOPS_E_INVAL, "null plan");
  SG_CUDA(cudaSetDevice(p->ctx->device));
  SG_CUDA(cudaGraphLaunch(p->exec, stream ? (cudaStream_t)stream : p->ctx->stream));
  return SIGOPS_OK;
}

void sigops_mixed_plan_destroy(sigops_plan* p) {
  if (!p) return;
  cudaSetDevice(p->ctx->device);
  if (p->exec) cudaGraphExecDestroy(p->exec);
  if (p->graph) cudaGraphDestroy(p->graph);
  delete p;
}

int sigops_set_variant(sigops_ctx* ctx, int kernel, int variant) {
  sigops_ctx* c = resolve(ctx);
  if (!c) return SIGOPS_E_NODEV;
  std::lock_guard<std::mutex> g(c->mu);
  SG_CUDA(cudaSetDevice(c->device));
  return set_variant(c, kernel, variant);
}

int sigops_get_variant(sigops_ctx* ctx, int kernel, int* variant, int* grid, int* block) {
  sigops_ctx* c = resolve(ctx);
  if (!c) return SIGOPS_E_NODEV;
  if (kernel >= 0 && kernel < 3) {
    if (variant) *variant = c->variant[kernel];
    if (grid) *grid = c->grid[kernel];
    if (block) *block = plain_variant_block(c->variant[kernel]);
    return SIGOPS_OK;
  }
  if (kernel == 3) {
    if (variant) *variant = c->batched_variant;
    if (grid) *grid = c->batched_grid;
    if (block) *block = batched_variant_block(c->batched_variant);
    return SIGOPS_OK;
  }
  return fail(SIGOPS_E_INVAL, "kernel id %d out of range", kernel);
}

int sigops_workload_sign_ecdsa(sigops_ctx* ctx, int curve, const uint8_t* d_secrets, const uint8_t* d_nonces, const uint8_t* d_msgs, size_t n,
                               uint8_t* d_sigs, uint8_t* d_pubkeys, uint8_t* d_status, void* stream) {
  if (curve != SIGOPS_SECP256K1 && curve != SIGOPS_SECP256R1) return fail(SIGOPS_E_INVAL, "ECDSA curve expected");
  if (n == 0) return SIGOPS_OK;
  if (!d_secrets || !d_nonces || !d_msgs || !d_sigs || !d_pubkeys || !d_status) return fail(SIGOPS_E_INVAL, "null device buffer");
  sigops_ctx* c = resolve(ctx);
  if (!c) return SIGOPS_E_NODEV;
  std::lock_guard<std::mutex> g(c->mu);
  SG_CUDA(cudaSetDevice(c->device));
  SG_CUDA(launch_sign_ecdsa(curve, d_secrets, d_nonces, d_msgs, n, c->d_gtab[curve], d_sigs, d_pubkeys, d_status, c->d_err, c->grid[curve],
                            stream ? (cudaStream_t)stream : c->stream));
  return SIGOPS_OK;
}

int sigops_workload_sign_ed25519(sigops_ctx* ctx, const uint8_t* d_seeds, const uint8_t* d_msgs, size_t n, uint8_t* d_sigs, uint8_t* d_pks,
                                 void* stream) {
  if (n == 0) return SIGOPS_OK;
  if (!d_seeds || !d_msgs || !d_sigs || !d_pks) return fail(SIGOPS_E_INVAL, "null device buffer");
  sigops_ctx* c = resolve(ctx);
  if (!c) return SIGOPS_E_NODEV;
  std::lock_guard<std::mutex> g(c->mu);
  SG_CUDA(cudaSetDevice(c->device));
  SG_CUDA(launch_sign_ed(d_seeds, d_msgs, n, c->d_gtab[2], d_sigs, d_pks, c->d_err, c->grid[2], stream ? (cudaStream_t)stream : c->stream));
  return SIGOPS_OK;
}

int sigops_sync(sigops_ctx* ctx) {
  sigops_ctx* c = resolve(ctx);
  if (!c) return SIGOPS_E_NODEV;
  std::lock_guard<std::mutex> g(c->mu);
  SG_CUDA(cudaSetDevice(c->device));
  SG_CUDA(cudaDeviceSynchronize());
  return check_device_errors(c);
}

int sigops_probe_mul(sigops_ctx* ctx, int form, double* rate) {
  if (!rate || form < 0 || form > 3) return fail(SIGOPS_E_INVAL, "bad probe form %d or null output", form);
  sigops_ctx* c = resolve(ctx);
  if (!c) return SIGOPS_E_NODEV;
  std::lock_guard<std::mutex> g(c->mu);
  SG_CUDA(cudaSetDevice(c->device));
  uint32_t* d_out = nullptr;
  SG_CUDA(cudaMalloc(&d_out, 16));
  const int block = 256, grid = c->num_sms * 8;
  const uint32_t iters = 4096;
  cudaEvent_t a, b;
  SG_CUDA(cudaEventCreate(&a));
  SG_CUDA(cudaEventCreate(&b));
  SG_CUDA(launch_mul_probe(form, d_out, 16, grid, block, c->stream));  // warm-up
  SG_CUDA(cudaEventRecord(a, c->stream));
  SG_CUDA(launch_mul_probe(form, d_out, iters, grid, block, c->stream));
  SG_CUDA(cudaEventRecord(b, c->stream));
  SG_CUDA(cudaEventSynchronize(b));
  float ms = 0;
  SG_CUDA(cudaEventElapsedTime(&ms, a, b));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(d_out);
  const double per_iter = form == 3 ? 8.0 * 8.0 : 8.0 * 16.0;
  *rate = (double)grid * block * iters * per_iter / (ms * 1e-3);
  return SIGOPS_OK;
}

int sigops_probe_imad(sigops_ctx* ctx, double* rate) { return sigops_probe_mul(ctx, 0, rate); }

int sigops_probe_k1_lanes(sigops_ctx* ctx, int lanes, int block, const uint8_t* d_sigs, const uint8_t* d_msgs, size_t n, uint8_t* d_out,
                          uint8_t* d_status, float* ms) {
  if ((lanes != 1 && lanes != 2) || block < 0 || block > 256 || block % 32 || !d_sigs || !d_msgs || !d_out || !d_status || !ms || n == 0)
    return fail(SIGOPS_E_INVAL, "sigops_probe_k1_lanes: bad arguments");
  auto misaligned = [](const void* p) { return ((uintptr_t)p & 15u) != 0; };
  if (misaligned(d_sigs) || misaligned(d_msgs) || misaligned(d_out)) return fail(SIGOPS_E_INVAL, "device buffers must be 16-byte aligned");
  sigops_ctx* c = resolve(ctx);
  if (!c) return SIGOPS_E_NODEV;
  std::lock_guard<std::mutex> g(c->mu);
  SG_CUDA(cudaSetDevice(c->device));
  cudaEvent_t a, b;
  SG_CUDA(cudaEventCreate(&a));
  SG_CUDA(cudaEventCreate(&b));
  SG_CUDA(launch_k1_lanes(lanes, d_sigs, d_msgs, n, block, c->d_gtab[0], d_out, d_status, c->stream));  // warm-up
  SG_CUDA(cudaEventRecord(a, c->stream));
  SG_CUDA(launch_k1_lanes(lanes, d_sigs, d_msgs, n, block, c->d_gtab[0], d_out, d_status, c->stream));
  SG_CUDA(cudaEventRecord(b, c->stream));
  SG_CUDA(cudaEventSynchronize(b));
  SG_CUDA(cudaEventElapsedTime(ms, a, b));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return SIGOPS_OK;
}

int sigops_probe_phase(sigops_ctx* ctx, int sync, const uint8_t* d_sigs, const uint8_t* d_msgs, size_t n, uint8_t* d_out,
                       uint8_t* d_status, uint64_t* d_times, float* ms) {
  if ((sync != 0 && sync != 1) || !d_sigs || !d_msgs || !d_out || !d_status || !d_times || !ms || n == 0)
    return fail(SIGOPS_E_INVAL, "sigops_probe_phase: bad arguments");
  auto misaligned = [](const void* p) { return ((uintptr_t)p & 15u) != 0; };
  if (misaligned(d_sigs) || misaligned(d_msgs) || misaligned(d_out) || ((uintptr_t)d_times & 7u))
    return fail(SIGOPS_E_INVAL, "device buffers must be 16-byte aligned (times: 8)");
  sigops_ctx* c = resolve(ctx);
  if (!c) return SIGOPS_E_NODEV;
  std::lock_guard<std::mutex> g(c->mu);
  SG_CUDA(cudaSetDevice(c->device));
  unsigned long long* counter = nullptr;
  SG_CUDA(dev_alloc((void**)&counter, sizeof(unsigned long long)));
  cudaEvent_t a = nullptr, b = nullptr;
  cudaError_t e = cudaEventCreate(&a);
  if (e == cudaSuccess) e = cudaEventCreate(&b);
  if (e == cudaSuccess) e = cudaMemsetAsync(counter, 0, sizeof(unsigned long long), c->stream);
  if (e == cudaSuccess) e = cudaEventRecord(a, c->stream);
  if (e == cudaSuccess)
    e = launch_k1_phase(sync != 0, d_sigs, d_msgs, n, c->d_gtab[0], d_out, d_status, counter, (unsigned long long*)d_times, c->num_sms,
                        c->stream);
  if (e == cudaSuccess) e = cudaEventRecord(b, c->stream);
  if (e == cudaSuccess) e = cudaEventSynchronize(b);
  if (e == cudaSuccess) e = cudaEventElapsedTime(ms, a, b);
  if (a) cudaEventDestroy(a);
  if (b) cudaEventDestroy(b);
  dev_free(counter);
  if (e != cudaSuccess) return fail(SIGOPS_E_CUDA, "sigops_probe_phase: %s", cudaGetErrorString(e));
  return SIGOPS_OK;
}

int sigops_device_info(sigops_ctx* ctx, int* num_sms, int* g1, int* g2, int* g3) {
  sigops_ctx* c = resolve(ctx);
  if (!c) return SIGOPS_E_NODEV;
  (void)0;
  if (num_sms) *num_sms = c->num_sms;
  if (g1) *g1 = c->grid[0];
  if (g2) *g2 = c->grid[1];
  if (g3) *g3 = c->grid[2];
  return SIGOPS_OK;
}

int sigops_test_field(sigops_ctx* ctx, int field, int op, const uint8_t* a, const uint8_t* b, uint8_t* out, size_t n) {
  if (field < 0 || field > 5 || op < 0 || op > 5 || !a || !b || !out) return fail(SIGOPS_E_INVAL, "bad field test arguments");
  if (n == 0) return SIGOPS_OK;
  sigops_ctx* c = resolve(ctx);
  if (!c) return SIGOPS_E_NODEV;
  std::lock_guard<std::mutex> g(c->mu);
  SG_CUDA(cudaSetDevice(c->device));
  int rc = ensure_buffers(c, n * 32 * 4);
  if (rc) return rc;
  uint8_t* da = c->d_buf;
  uint8_t* db = da + n * 32;
  uint8_t* dout = db + n * 32;
  SG_CUDA(cudaMemcpyAsync(da, a, n * 32, cudaMemcpyHostToDevice, c->stream));
  SG_CUDA(cudaMemcpyAsync(db, b, n * 32, cudaMemcpyHostToDevice, c->stream));
  SG_CUDA(cudaMemsetAsync(dout, 0, n * 64, c->stream));
  SG_CUDA(launch_field_test(field, op, da, db, dout, (int)n, c->stream));
  SG_CUDA(cudaMemcpyAsync(out, dout, n * 64, cudaMemcpyDeviceToHost, c->stream));
  SG_CUDA(cudaStreamSynchronize(c->stream));
  return SIGOPS_OK;
}

int sigops_test_wait_expiry(sigops_ctx* ctx, uint32_t max_polls) {
  if (max_polls == 0 || max_polls > (1u << 16)) return fail(SIGOPS_E_INVAL, "max_polls must be in [1, 65536]");
  sigops_ctx* c = resolve(ctx);
  if (!c) return SIGOPS_E_NODEV;
  std::lock_guard<std::mutex> g(c->mu);
  SG_CUDA(cudaSetDevice(c->device));
  SG_CUDA(launch_wait_expiry(max_polls, c->d_err, c->stream));
  return check_device_errors(c);
}

int sigops_test_fail_allocations(int count) { return g_fail_allocs.exchange(count < 0 ? 0 : count); }

int sigops_test_sha512(sigops_ctx* ctx, const uint8_t* in, uint8_t* out, size_t n) {
  if (!in || !out) return fail(SIGOPS_E_INVAL, "null buffer");
  if (n == 0) return SIGOPS_OK;
  sigops_ctx* c = resolve(ctx);
  if (!c) return SIGOPS_E_NODEV;
  std::lock_guard<std::mutex> g(c->mu);
  SG_CUDA(cudaSetDevice(c->device));
  int rc = ensure_buffers(c, n * 160);
  if (rc) return rc;
  SG_CUDA(cudaMemcpyAsync(c->d_buf, in, n * 96, cudaMemcpyHostToDevice, c->stream));
  SG_CUDA(launch_sha512_test(c->d_buf, c->d_buf + n * 96, (int)n, c->stream));
  SG_CUDA(cudaMemcpyAsync(out, c->d_buf + n * 96, n * 64, cudaMemcpyDeviceToHost, c->stream));
  SG_CUDA(cudaStreamSynchronize(c->stream));
  return SIGOPS_OK;
}

}  // extern "C"
